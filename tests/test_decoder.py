"""Setup-time decoding on the host (no GPU): every model the configs build
decodes; unimplemented or malformed programs are hard errors naming the
solver, row, opcode and position (there is no CPU fallback)."""
import numpy as np
import pytest

import ophelpers as A
from gbhsolve import configs, engine, model


def _err(hs):
    with pytest.raises(engine.EngineError) as ei:
        engine.validate(hs)
    return ei.value


def test_configs_decode():
    assert engine.validate([model.build(configs.ap_verify(8))]) == (8, 1)
    hs, _ = configs.cables_replicated(64, gk_dend=36.0)
    assert engine.validate(hs) == (64, 1)
    one = model.build(configs.cables(5, gk_dend=36.0, method=model.CRANK)[0])
    n, t = engine.validate([one])
    assert n == 5
    trees = [model.build(m) for m in configs.random_trees(30, size_range=(8, 40), seed=1)]
    assert engine.validate(trees)[0] == 30
    ms, _ = configs.hh_network(20, p_conn=0.2)
    assert engine.validate([model.build(m) for m in ms]) == (20, 1)


def _hh():
    c = A.Compt(-2e-10, 1e-10, 2.0, 1.01, 3e8, -0.06)
    c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[0.05, 1e-8]).op(A.IPOL1V, 0, 3, chips=[0.1]).op(A.ADD_CURR, giv=3)
    return c


def test_unknown_opcode_is_rejected():
    c = _hh()
    c.ops.insert(1, 7777)
    e = _err([A.solver([c], A.tables(12, 20))])
    assert e.code == -2 and e.opcode == 7777 and e.row == 0 and e.position == 2


def test_unknown_conductance_opcode_is_rejected():
    c = A.Compt(-2e-10, 1e-10, 2.0, 1.01, 3e8, -0.06)
    c.op(A.NEWVOLT).op(A.CHAN_EK, 4099, chips=[0.05, 1e-8])
    e = _err([A.solver([c], A.tables(12, 20))])
    assert e.code == -2 and e.opcode == 4099


def test_store_op_without_storemode_is_rejected():
    c = _hh()
    c.op(A.STORE_ALLI, 0)
    e = _err([A.solver([c], A.tables(12, 20))])
    assert e.code == -1 and e.opcode == A.STORE_ALLI


@pytest.mark.parametrize("token", [3, 4, 5])
def test_symmetric_token_with_index_out_of_range_is_rejected(token):
    """Symmetric-compartment tokens are run as written; one whose ravals
    index lies outside the solver's ravals[] is a funcs error."""
    h = A.solver([_hh(), _hh()], A.tables(12, 20), parents=[1, -1])
    f = list(h.funcs)
    f[0:0] = [token, 10 ** 6] if token != 5 else [token, 0, 10 ** 6]
    h.funcs = np.array(f, np.int32)
    e = _err([h])
    assert e.code == -3 and e.opcode == token


def test_truncated_chip_is_rejected():
    h = A.solver([_hh()], A.tables(12, 20))
    h.chip = h.chip[:4]
    e = _err([h])
    assert e.code == -1


def test_error_names_the_solver():
    good = A.solver([_hh()], A.tables(12, 20))
    c = _hh()
    c.ops.append(9999)
    bad = A.solver([c], A.tables(12, 20))
    e = _err([good, good, bad])
    assert e.solver == 2


def _syn_solver(order):
    """One compartment with two synchans whose constant sets (stablist
    entries 0 and 4 of its own stablist) are used in the given order."""
    c = A.Compt(-2e-10, 1e-10, 2.0, 1.01, 3e8, -0.06)
    for stab in order:
        c.op(A.CHAN_EK, chips=[0.0, 1e-9]).op(A.SYN2, stab, -1, 1, chips=[0.4, 0.7], giv=3)
    sa = [0.99, 9.5e-5, 0.98, 9.9e-5 / 2e-5]
    sb = [0.95, 8.0e-5, 0.97, 9.0e-5 / 2e-5]
    return A.solver([c], A.tables(12, 20), stablist=sa + sb)


def test_parallel_decode_merges_synchan_constants():
    """Large batches decode in chunks on several threads; the chunks'
    synchan constant sets are renumbered into the batch's first-come order
    and the programs regrouped. Solvers using the sets in opposite orders
    are two program types however the batch is chunked."""
    from gbhsolve import engine
    n = 4096
    hs = [_syn_solver([0, 4])] * (n // 2) + [_syn_solver([4, 0])] * (n // 2)
    assert engine.validate(hs) == (n, 2)
    assert engine.validate(hs[n // 2:]) == (n // 2, 1)


def test_parallel_decode_reports_first_error_in_solver_order():
    good = _syn_solver([0, 4])
    bad = A.solver([_hh()], A.tables(12, 20))
    bad.chip = bad.chip[:4]
    worse = _syn_solver([0, 4])
    worse.ops = worse.ops.copy()
    worse.ops[1] = 7777
    hs = [good] * 4096
    hs[1500], hs[3900] = bad, worse
    e = _err(hs)
    assert e.solver == 1500 and e.code == -1
