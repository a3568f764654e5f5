"""Batched form: many uneven instances in one solver (cfd2d_batch_create).

Each instance's state after the batched steps must equal its own
single-instance solve bit for bit (the kernels are the single-instance ones
over the union mesh; each instance keeps its own time step), whatever launch
shapes the autotuner picks.
"""
import os

import numpy as np
import pytest

from cfd2d import cases
from test_oracle_golden import bits_equal

pytestmark = pytest.mark.gpu


def _batch(capi, tmp_path, insts):
    paths = []
    for k, (t, m, _) in enumerate(insts):
        d = tmp_path / f"i{k}"
        d.mkdir()
        paths.append(cases.write_task(t, m, str(d)))
    b = capi.Batch(paths, meshes=[m for _, m, _ in insts])
    U = np.concatenate([U0 for _, _, U0 in insts], axis=1)
    b.set_state(U, reset_time_step=True)
    return b, paths


@pytest.mark.parametrize("precision", [None, "MIXED"])
def test_batch_equals_single_solves(capi, tmp_path, precision):
    insts = cases.batched_vortices(7, min_cells=150, max_cells=3000, steps=15, precision=precision)
    b, paths = _batch(capi, tmp_path, insts)
    assert b.info.n_instances == 7
    b.step(15)
    Ub = b.state()
    for k, (t, m, U0) in enumerate(insts):
        s = capi.Solver(paths[k], mesh=m)
        s.set_state(U0, reset_time_step=True)
        off, nc, tau, _ = b.instance(k)
        assert nc == m.n_cells and tau == s.tau
        s.step(15)
        assert bits_equal(Ub[:, off:off + nc], s.state())


def _sub(p, name):
    d = p / name
    d.mkdir()
    return d


def test_autotuned_shapes_keep_results(capi, tmp_path):
    insts = cases.batched_vortices(5, min_cells=2000, max_cells=20000, steps=5)
    a, _ = _batch(capi, _sub(tmp_path, "a"), insts)
    js = str(tmp_path / "tuning.json")
    a.autotune(js)
    assert os.path.exists(js) and '"flux"' in open(js).read()
    b, _ = _batch(capi, _sub(tmp_path, "b"), insts)
    b.load_tuning(js)
    a.step(5); b.step(5)
    ref, _ = _batch(capi, _sub(tmp_path, "c"), insts)
    ref.step(5)
    assert bits_equal(a.state(), ref.state()) and bits_equal(b.state(), ref.state())
