"""Failure detection without a GPU fault: every wait on the device is
bounded and every failure the kernels detect comes back as a status word
that the next synchronous call turns into an error, with the context still
usable.

* A neuron whose Vm becomes NaN or infinite (planted on the host through
  gbh_set_state) is reported by gbh_run as GBH_ERR_DEVICE, on every kernel
  path (interpreted, specialised, wide tiles, stack elimination, mixed).
* The grid barrier of the cooperative multi-step launch gives up after its
  poll limit when the arrivals it waits for never come (a test program waits
  for a block that is never launched), raises ST_BARRIER and returns.
"""
import os
import subprocess

import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "genesis-2.4_gb300", "csrc")
ST_BARRIER, ST_NONFINITE = 8, 16


@pytest.mark.parametrize("kw", [dict(jit=False, wide_min=-1), dict(jit=True, wide_min=-1),
                                dict(jit=False, wide_min=32), dict(jit=True, wide_min=0, precision=1)])
def test_nonfinite_vm_is_reported(gpu_engine, kw):
    hs = [model.build(m) for m in configs.random_trees(40, size_range=(8, 120), seed=31)]
    eng = gpu_engine.Engine(hs, steps_per_launch=10, **kw)
    eng.run(20)
    st = eng.get_state()
    vm = [v.copy() for v in st["vm"]]
    vm[17][3] = np.nan                     # one compartment of one neuron
    eng.set_state(vm=vm)
    with pytest.raises(RuntimeError, match="NaN or infinite"):
        eng.run(5)
    eng.close()
    # a fresh engine on the same device still runs
    ok = gpu_engine.Engine(hs[:4], steps_per_launch=10)
    ok.run(10)
    assert np.all(np.isfinite(ok.vm()))
    ok.close()


def test_finite_run_reports_nothing(gpu_engine):
    hs = [model.build(m) for m in configs.random_trees(40, size_range=(8, 120), seed=32)]
    eng = gpu_engine.Engine(hs, steps_per_launch=10, wide_min=-1)
    eng.run(200)
    assert np.all(np.isfinite(eng.vm()))
    eng.close()


def test_grid_barrier_wait_runs_out(tmp_path):
    exe = str(tmp_path / "barrier_timeout")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-I", CSRC,
                    os.path.join(HERE, "cuda", "barrier_timeout.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    f = out.stdout.split()
    status, gave_up, ms, ctx = int(f[1]), int(f[3]), float(f[5]), int(f[9])
    assert status & ST_BARRIER
    assert gave_up == 2               # both launched blocks gave up and returned
    assert ctx == 1                   # a later kernel ran normally
    assert ms < 60_000
