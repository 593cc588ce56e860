"""The reference's own GPU arm: its CUDA backend (genesis/src/hines/cuda/,
rebuilt for sm_103a by `make -C oracle cuda-ref`) stepping the cables
workload of 1,000 neurons x 16 compartments as one hsolve, 200 steps of
backward Euler at dt = 20 us, in the per-step mode hines.c uses under
USE_CUDA (per step: Vm to the device, the FP32 channel kernel, (rhs, diag)
back, then the reference's CPU Hines solve).

BENCHMARK INFRASTRUCTURE: run as its own process (`python oracle/ref_cuda.py`),
so a failure of the reference's GPU code cannot take the caller down; prints
one JSON line: the run's wall-clock rate, the reference's own kernel time
(its CUDA-event profile), and max |dVm| of its FP32 result against the FP64
oracle on the same model. Its multi-step mode is not run: its tree kernel
reads results[-2] for the first tree (cuda_channel.cuh:498-501), an
out-of-bounds read.
"""
import ctypes as C
import io
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "genesis-2.4_gb300"))

LIB = os.path.join(HERE, "_ref", "libhcuda_ref.so")
NEURONS, NCOMP, NSTEPS = 1000, 16, 200


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "cuda-ref"], check=True, stdout=subprocess.DEVNULL)


def measure() -> dict:
    import numpy as np
    import pyoracle
    from gbhsolve import configs, model

    pyoracle.ensure_built()
    h = model.build(configs.cables(NEURONS)[0])
    ref = pyoracle.Solver(h)
    ref.run(NSTEPS)                        # FP64 oracle (the reference's CPU step, bit for bit)
    s = pyoracle.Solver(h)
    lib = C.CDLL(LIB)
    lib.rch_perstep.argtypes = [C.POINTER(pyoracle.OrcSolver), C.c_int, C.POINTER(C.c_double)]
    wall = C.c_double(0.0)
    # the reference prints its profile on stdout: capture the file descriptor
    sys.stdout.flush()
    saved = os.dup(1)
    with tempfile.TemporaryFile(mode="w+b") as tmp:
        os.dup2(tmp.fileno(), 1)
        try:
            rc = lib.rch_perstep(C.byref(s.s), NSTEPS, C.byref(wall))
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        tmp.seek(0)
        text = tmp.read().decode(errors="replace")
    if rc != 0:
        return {"unavailable": "the reference's CUDA backend refused or failed: " + text.strip()[-300:]}
    m = re.search(r"kernel total\s*:\s*([0-9.]+) ms\s*\(([0-9.]+) us/step\)", text)
    ncs = NEURONS * NCOMP * NSTEPS
    out = {
        "workload": "cables-1k-x16: 1,000 neurons x 16 compartments as one hsolve, %d steps, dt 20 us, "
                    "backward Euler" % NSTEPS,
        "code": "genesis/src/hines/cuda/cuda_hsolve.c + cuda_backend.cu + cuda_channel.cuh, built for sm_103a, "
                "per-step mode (FP32 channel kernel on the GPU; the reference's CPU Hines solve)",
        "wall_ms": wall.value,
        "value": ncs / (wall.value * 1e-3),
        "unit": "compartment-steps/s",
        "max_abs_dvm_vs_fp64_oracle_V": float(np.max(np.abs(s.vm - ref.vm))),
    }
    if m:
        out["kernel_ms"] = float(m.group(1))
        out["kernel_us_per_step"] = float(m.group(2))
    return out


if __name__ == "__main__":
    try:
        build()
        res = measure()
    except Exception as ex:  # noqa: BLE001 -- reported, not raised: the caller records it
        res = {"unavailable": "%s: %s" % (type(ex).__name__, ex)}
    print(json.dumps(res), flush=True)
