"""astrea_step_host: a step whose input and output live in host memory.

For callers that keep the grid on the host between steps (as the reference's
core_run does): the state is copied in, stepped, and left in host memory.  With
page-locked output and an SSP-RK (2,2)/(3,3)/(4,3) integrator the last combining
sweep writes the result to the host itself; otherwise the state is copied out
after the step.  Either way the result must equal the device-only step bit for
bit in FP64 (the same kernels), over consecutive steps that feed the output
back as the next input.
"""

import numpy as np
import pytest
import torch

import bench
from astrea_gb300.solver import RunConfig, Solver

pytestmark = pytest.mark.gpu


def pair(cfg, w):
    a, b = Solver(cfg), Solver(cfg)
    for s in (a, b):
        s.initialise(w)
        s.reset_clock()
    return a, b


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("integrator", ["ssprk33", "euler"])
def test_host_step_equals_device_step(pinned, integrator):
    from dataclasses import replace
    n = 128
    cfg = replace(bench.run_config(n, 64), integrator=integrator)
    ref, s = pair(cfg, bench.shear_layer(n))
    host = s.state.cpu()
    if pinned:
        host = host.pin_memory()
    for _ in range(3):
        ref.step(1, graph=False)
        s.step_host(host, host)
        torch.cuda.synchronize()
        assert torch.equal(host, ref.state.cpu())
        assert torch.equal(s.state, ref.state)
    assert s.clock() == ref.clock()


def test_host_step_fp32_and_separate_buffers():
    n = 256
    cfg = bench.run_config(n, 32)
    ref, s = pair(cfg, bench.shear_layer(n))
    h_in = s.state.cpu().pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    for _ in range(2):
        ref.step(1, graph=True)
        s.step_host(h_in, h_out)
        torch.cuda.synchronize()
        assert torch.equal(h_out, ref.state.cpu())
        h_in.copy_(h_out)
