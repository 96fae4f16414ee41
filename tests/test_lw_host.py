"""Lax-Wendroff (num_methods/solvers.py:79-88): what the reference's coefficient is, on the CPU.

The reference's LW flux is LLF's form with the per-interface coefficient
(sound speed)^2 / max|lambda|, where the 'sound speed' is
``np.unique(characteristics, axis=-1)[..., 1]``: the second of the eigenvalue
*columns* of the whole interface array after a lexicographic sort.  Which wave
that column holds is decided by the first interface where the candidate
columns differ.  tests/golden/lw_columns.npz (made from the reference by
make_golden.py:lw_columns) records the column per step of three 1D runs; these
tests pin what it is, and pin the oracle, whose 'lapack' mode applies the
reference's rule and whose 'analytic' mode (the kernels' closed form) takes
the entropy-wave eigenvalue v_n:

* Sod with PPM: the column is v_n at the start of every step, yet not in the
  later Runge-Kutta stages, so even there the closed form departs within the
  first step;
* Sod with PLM: the column is v_n on some steps and the zero eigenvalue of the
  B_n row on others (the velocity's sign at the first disturbed interface
  decides), so no per-interface formula reproduces the reference;
* a sine wave: the column is neither.

The kernels take v_n (the entropy wave the reference's comment names), so
their Lax-Wendroff parity is against the oracle's 'analytic' mode only.
"""

import json
import os

import numpy as np
import pytest

from oracle import stepper
from tests.golden_io import GOLDEN


@pytest.fixture(scope="module")
def cols():
    with np.load(os.path.join(GOLDEN, "lw_columns.npz")) as z:
        return {k: z[k] for k in z.files}


def steps(cols, tag):
    return json.loads(str(cols[f"{tag}_meta"]))["steps"]


def test_sod_ppm_column_is_the_entropy_wave_every_step(cols):
    for s in range(steps(cols, "sod_ppm")):
        assert np.array_equal(cols[f"sod_ppm_col_s{s}"], cols[f"sod_ppm_vn_s{s}"])
    assert np.max(np.abs(cols["sod_ppm_vn_s2"])) > .5  # a non-trivial velocity field by then


def test_sod_plm_column_switches_between_eigenvalues(cols):
    same, zero = [], []
    for s in range(steps(cols, "sod_plm")):
        col, vn = cols[f"sod_plm_col_s{s}"], cols[f"sod_plm_vn_s{s}"]
        same.append(bool(np.array_equal(col, vn)))
        zero.append(bool(np.all(col == 0) and np.max(np.abs(vn)) > .5))
    assert any(same) and any(zero), (same, zero)


def test_sine_column_is_neither(cols):
    col, vn = cols["sin_plm_col_s0"], cols["sin_plm_vn_s0"]
    assert not np.allclose(col, vn) and not np.all(col == 0)


def oracle_cfg(meta, eig):
    return stepper.OracleConfig(dim=1, scheme=meta["subgrid"], solver="lw", integrator="ssprk33", gamma=meta["gamma"],
                                bc=meta["boundary"], dx=meta["dx"], cfl=meta["cfl"], eig=eig, t_end=meta["t_end"])


@pytest.mark.parametrize("tag", ["sod_plm", "sod_ppm", "sin_plm"])
def test_oracle_lapack_mode_reproduces_reference_lw(cols, tag):
    meta = json.loads(str(cols[f"{tag}_meta"]))
    cfg = oracle_cfg(meta, "lapack")
    q, t, idx, order = cols[f"{tag}_q0"], 0.0, 1, [0]
    with np.errstate(all="ignore"):
        for s in range(meta["steps"]):
            q, t, idx, order, _ = stepper.step(q, cfg, t, idx, order)
            ref = cols[f"{tag}_q_{s + 1}"]
            assert np.max(np.abs(q - ref)) <= 1e-13 * np.max(np.abs(ref)), (tag, s)


@pytest.mark.parametrize("tag", ["sod_plm", "sod_ppm"])
def test_closed_form_departs_from_the_reference_within_the_first_step(cols, tag):
    """The first stage of the first step agrees (the column is v_n = 0 on the initial state);
    the later stages see a non-zero velocity and the reference's column is another wave."""
    meta = json.loads(str(cols[f"{tag}_meta"]))
    q0 = cols[f"{tag}_q0"]
    with np.errstate(all="ignore"):
        fl = {eig: stepper.evolve_space(q0, oracle_cfg(meta, eig), [0]) for eig in ("lapack", "analytic")}
        assert np.array_equal(fl["lapack"][0]["flux"], fl["analytic"][0]["flux"])
        q_a, *_ = stepper.step(q0, oracle_cfg(meta, "analytic"), 0.0, 1, [0])
    assert np.max(np.abs(q_a - cols[f"{tag}_q_1"])) > 1e-6
