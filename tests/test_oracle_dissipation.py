"""The oracle's PPM flattening and artificial viscosity act on the states the GPU parity cases use.

Both terms are parity-unpinned (the reference's code for them fails when
called); these checks make sure the parity cases in test_gpu_dissipation.py
exercise them: the flattening coefficient drops below 1 along both axes and the
viscous flux is non-zero on the 96^2 four-quadrant state.
"""

import numpy as np

from oracle import recon, stepper
from tests.test_gpu_dissipation import quadrants


def test_the_cases_exercise_both_terms():
    # the oracle flattens and adds viscosity on these initial states (so the tests above test something)
    n = 96
    w = quadrants(n, 35)
    oc = stepper.OracleConfig(dim=2, scheme="ppm", solver="hllc", integrator="ssprk33", gamma=1.4, bc="edge",
                              dx=1.0 / n, cfl=0.4, eig="analytic", t_end=1.0, flatten=True, viscosity=True)
    q = stepper.initialise(w, oc)
    wS = stepper.convert_conservative(q, oc, [0, 1])
    assert recon.flatten_coefficient(wS, 0, "edge").min() < 1.0
    assert recon.flatten_coefficient(wS.transpose(1, 0, 2), 1, "edge").min() < 1.0
    assert np.abs(stepper.artificial_viscosity(wS, q, 0, oc)).max() > 0.0
