"""SETUP of many hsolves on several processes (model.build_many,
model.build_generated): the arrays equal those of the one-process build
exactly, in order, and solvers with equal composite tables share one copy
of them. Random trees generated in ranges equal the whole set's."""
import dataclasses

import numpy as np

from gbhsolve import configs, model


def _same(a, b):
    for f in dataclasses.fields(a):
        u, v = getattr(a, f.name), getattr(b, f.name)
        if isinstance(u, np.ndarray):
            assert u.dtype == v.dtype and np.array_equal(u, v), f.name
        else:
            assert u == v, f.name


def test_random_trees_in_ranges_equal_the_whole_set():
    whole = configs.random_trees(40, size_range=(8, 30), seed=6)
    part = configs.random_trees(40, size_range=(8, 30), seed=6, start=17, stop=29)
    for m, p in zip(whole[17:29], part):
        _same(model.build(m), model.build(p))


def test_build_generated_and_build_many_equal_build():
    kw = dict(size_range=(8, 40), seed=8)
    ref = [model.build(m) for m in configs.random_trees(300, **kw)]
    gen = model.build_generated(configs.random_trees, 300, workers=2, chunk=64, **kw)
    many = model.build_many(configs.random_trees(300, **kw), workers=2, chunk=64)
    assert len(gen) == len(many) == 300
    for r, g, m in zip(ref, gen, many):
        _same(r, g)
        _same(r, m)
    assert len({id(g.tablist) for g in gen}) == 1
    assert len({id(m.tablist) for m in many}) == 1
