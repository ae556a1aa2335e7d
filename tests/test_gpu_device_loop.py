"""The Newton loop on the device (GPU): SweepX{0} as one CUDA graph launch
whose conditional WHILE nodes loop over the load steps and the Newton
iterations (mgpu_sweep_opts.device_loop).  The same kernels run in the same
order as the host-driven loop, so the states are bitwise those of the host
loop, with per-model convergence (batched models) and with the global test
(one model); a bounded iteration count ends in the reference's "no
convergence" error after the steps that converged.
"""
import math

import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceError, DeviceModel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()


def test_batched_models_per_component():
    params = W.batched_params(12, nel_range=(10, 60), seed=5)
    m, _, times = W.build_batched(params)
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    kw = dict(maxdx=1e-9, maxLl=math.inf, per_component=True)
    rc_h, xh, sh = dm.sweepx(0, times, st.time, list(st.X), **kw)
    rc_d, xd, sd = dm.sweepx(0, times, st.time, list(st.X), device_loop=True, **kw)
    dm.close()
    assert rc_h == 0 and rc_d == 0
    assert sd.nstep_done == sh.nstep_done == len(times)
    assert sd.niter_total == sh.niter_total
    assert np.array_equal(xd, xh)


def test_single_model_global_test_and_iteration_bound():
    m, times = W.cantilever(nel=20)
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    rc_h, xh, sh = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-9, maxLl=1e-5)
    rc_d, xd, sd = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-9, maxLl=1e-5, device_loop=True)
    assert rc_h == 0 and rc_d == 0 and sd.niter_total == sh.niter_total
    assert np.array_equal(xd, xh)
    # too few iterations: the host loop and the device loop stop at the same step
    rc_h, xh, sh = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-9, maxLl=1e-5, maxiter=4)
    rc_d, xd, sd = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-9, maxLl=1e-5, maxiter=4, device_loop=True)
    assert rc_h == rc_d != 0 and sd.nstep_done == sh.nstep_done and sd.fail_step == sh.fail_step
    with pytest.raises(DeviceError) as e:
        dm._check(rc_d)
    assert e.value.kind == "noconvergence" and "no convergence of step" in str(e.value)
    k = sd.nstep_done
    assert np.array_equal(xd[:k], xh[:k])
    dm.close()
