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


@pytest.mark.parametrize("precision", [None, "MIXED"])
def test_batch_adjoint_equals_single_adjoints(capi, tmp_path, precision):
    """The discrete adjoint over the union mesh: each instance's slice of dJ/dU0 and
    of dJ/d(boundary parameters) equals its own single-instance adjoint bit for bit
    (J of the batch is the sum of the instances' J)."""
    insts = cases.batched_vortices(3, min_cells=300, max_cells=2500, steps=6, flux="HLLC", precision=precision)
    b, paths = _batch(capi, tmp_path, insts)
    rng = np.random.default_rng(11)
    ws = [rng.uniform(0.0, 1.0, m.n_cells) for _, m, _ in insts]
    b.set_objective(0, np.concatenate(ws), 1.0)
    b.set_state(np.concatenate([U0 for _, _, U0 in insts], axis=1), reset_time_step=True)
    Jb = b.forward(6, 3)
    g, gb = b.backward()
    J = 0.0
    nb = 0
    for k, (t, m, U0) in enumerate(insts):
        s = capi.Solver(paths[k], mesh=m)
        s.set_objective(0, ws[k], 1.0)
        s.set_state(U0, reset_time_step=True)
        J += s.forward(6, 3)
        gk, gbk = s.backward()
        off, nc, _, _ = b.instance(k)
        assert bits_equal(g[:, off:off + nc], gk)
        assert bits_equal(gb[nb:nb + len(gbk)], gbk)
        nb += len(gbk)
    assert abs(Jb - J) <= 1e-14 * abs(J)
