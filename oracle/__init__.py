"""CPU oracle for astrea's per-step finite-volume update.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, and only as the checker (or the timed CPU
baseline), never as the thing that is measured or shipped.

The oracle restates, in NumPy, the arithmetic of the reference hot path
(mervyzr/astrea: ``functions/fv.py``, ``functions/constructor.py``,
``schemes/*.py``, ``num_methods/{limiters,solvers,mag_field,evolvers}.py``)
with the same floating-point operation order, so that in FP64 it agrees with
the reference bit for bit.  It is *pinned* against the reference itself:
``tests/golden/make_golden.py`` imports the reference (only where it is
available) and writes golden input/output vectors that ``tests/`` compare the
oracle against.

Formulation.  The reference pads every intermediate array with
``np.pad(mode=edge|wrap)`` and slices it.  Here every out-of-range access to an
intermediate ``X`` is written as an explicit gather ``X[bc(i + s)]`` with
``bc`` = clamp (outflow) or modulo (periodic) applied to *that* intermediate.
This is the same "per-intermediate boundary" rule the CUDA kernels implement,
and it is what makes outflow tiles differ from a single ghost fill.

Modules:
  fvcore   - boundary gathers, masked divide, prim<->cons, 4th-order
             conversions, physical flux, interface averages, wave speeds
  recon    - PLM (minmod / superbee), PPM (McCorquodale-Colella limiter),
             WENO-3/5/7
  riemann  - LLF, LW, HLLC, HLLD interface fluxes
  ct       - constrained-transport pieces for 2D MHD
  stepper  - configuration, evolve_space / evolve_time, run-to-t_end driver
"""

from . import fvcore, recon, riemann, ct, stepper  # noqa: F401
from .stepper import OracleConfig, evolve_space, evolve_time, run, step, initialise  # noqa: F401
