"""The per-program kernels the engine generates at setup compile for sm_103a
(NVRTC, no GPU needed) for every kind of program the configs produce."""
import ctypes as C
import os

import pytest

from gbhsolve import build, configs, engine, model

CSRC = os.path.join(os.path.dirname(build.ROOT), "genesis-2.4_gb300", "csrc")


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    pytest.skip("libnvrtc not available")


def compile_sm103a(src, fp64_exact):
    lib = _nvrtc()
    prog = C.c_void_p()
    heads = ["gbh_internal.h", "gbh_df.cuh", "gbh_devfn.cuh"]
    texts = [open(os.path.join(build.CSRC, h)).read().encode() for h in heads]
    texts += [b"", build.STDINT_STUB.encode()]
    names = [h.encode() for h in heads] + [b"cuda_runtime.h", b"stdint.h"]
    arr_t = (C.c_char_p * len(texts))(*texts)
    arr_n = (C.c_char_p * len(names))(*names)
    assert lib.nvrtcCreateProgram(C.byref(prog), src.encode(), b"gbh_jit.cu", len(texts), arr_t, arr_n) == 0
    opts = [b"--gpu-architecture=sm_103a", b"--std=c++17", b"-default-device"]
    if fp64_exact:
        opts.append(b"--fmad=false")
    rc = lib.nvrtcCompileProgram(prog, len(opts), (C.c_char_p * len(opts))(*opts))
    n = C.c_size_t()
    lib.nvrtcGetProgramLogSize(prog, C.byref(n))
    log = C.create_string_buffer(n.value + 1)
    lib.nvrtcGetProgramLog(prog, log)
    lib.nvrtcDestroyProgram(C.byref(prog))
    return rc, log.value.decode(errors="replace")


def _models():
    yield "cables-uniform", configs.cables_replicated(4, gk_dend=36.0)[0]
    yield "cables-passive", configs.cables_replicated(4, gk_dend=0.0)[0]   # static rows kept across steps
    yield "single-hsolve", [model.build(configs.cables(3, gk_dend=36.0, method=model.CRANK)[0])]
    yield "trees-ca", [model.build(m) for m in configs.random_trees(3, size_range=(12, 12), seed=4)]
    ms, _ = configs.hh_network(6, p_conn=0.5)
    yield "network", [model.build(m) for m in ms]


@pytest.mark.parametrize("compact", [0, 1, 2])
@pytest.mark.parametrize("prec", [engine.PREC_FP64, engine.PREC_MIXED])
@pytest.mark.parametrize("name,hs", list(_models()))
def test_generated_kernel_compiles(name, hs, prec, compact):
    src = engine.jit_source(hs, precision=prec, type_index=0, compact=compact)
    assert "gbh_jit" in src
    rc, log = compile_sm103a(src, prec == engine.PREC_FP64)
    assert rc == 0, log[:4000]


def test_compact_form_loops_identical_compartments():
    """The identical dendrites of a cable (all but the first, which holds the
    K channel's Ek) become one loop in the compact form; the unrolled form
    has none."""
    hs = configs.cables_replicated(4, gk_dend=36.0)[0]
    loop = engine.jit_source(hs, precision=engine.PREC_MIXED, compact=True)
    flat = engine.jit_source(hs, precision=engine.PREC_MIXED, compact=False)
    assert "for (int s = 1; s < 15; ++s)" in loop
    assert "for (int s = " not in flat
    assert len(loop) < len(flat) / 3


def test_shared_rows_form_keeps_rows_out_of_registers():
    """The unrolled form with shared-memory rows declares no D/R register
    arrays; its fused elimination and back-substitution address the columns."""
    hs = configs.cables_replicated(4, gk_dend=36.0)[0]
    regs = engine.jit_source(hs, precision=engine.PREC_MIXED, compact=0)
    cols = engine.jit_source(hs, precision=engine.PREC_MIXED, compact=2)
    assert "double D[16], R[16], T[16]" in regs
    assert "double D[16]" not in cols and "double T[16]" in cols
    assert "Dc[(15) * 32]" in cols and "Rc[480]" in cols
    assert "dynamic_smem_size" in cols and "dynamic_smem_size" not in regs


@pytest.mark.parametrize("prec", [engine.PREC_FP64, engine.PREC_MIXED])
def test_static_rows_only_where_rows_are_passive(prec):
    """The unrolled register form keeps the factors of the passive rows below
    the first compartment with channels: passive dendrites get the kept-factor
    phase (15 of 16 rows), active dendrites and the looped forms do not."""
    passive = configs.cables_replicated(4, gk_dend=0.0)[0]
    active = configs.cables_replicated(4, gk_dend=36.0)[0]
    src = engine.jit_source(passive, precision=prec, type_index=0, compact=0)
    assert src.count("kept factors") == 15 and "v.tgen[t] = sgen" in src
    for hs, compact in ((active, 0), (passive, 1), (passive, 2)):
        assert "kept factors" not in engine.jit_source(hs, precision=prec, type_index=0, compact=compact)
