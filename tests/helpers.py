"""Comparison helpers shared by the parity tests."""
from __future__ import annotations

import numpy as np


def gpu_sim_for_scene(scene, max_particles: int = 0, sdf=None):
    from fluidsph.sim import SphSimulation3DGrid
    sim = SphSimulation3DGrid(scene.particles, scene.sph, scene.geom, max_particles, sdf)
    sim.update_gravity(scene.gravity)
    sim.set_pcisph_iterations(scene.iterations)
    if scene.rigid is not None:
        sim.update_rigid_body(scene.rigid)
    return sim


def assert_same_floats(a: np.ndarray, b: np.ndarray, what: str = "") -> None:
    """Bit-exact float comparison (== with NaN == NaN; +0 == -0)."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    if not same.all():
        idx = np.argwhere(~same)
        i = tuple(idx[0])
        raise AssertionError(
            f"{what}: {int((~same).sum())} of {a.size} values differ; first at {i}: "
            f"{a[i]!r} vs {b[i]!r} (max abs diff {np.nanmax(np.abs(a - b))})")


def assert_close_rel(a, b, rtol: float, what: str = "", floor: float = 0.0) -> None:
    """|a - b| <= rtol * max(|b|, floor) element-wise."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    err = np.abs(a - b)
    lim = rtol * np.maximum(np.abs(b), floor)
    bad = err > lim
    if bad.any():
        i = np.argmax(err - lim)
        raise AssertionError(f"{what}: {int(bad.sum())} values beyond rtol {rtol}; worst "
                             f"{a.flat[i]!r} vs {b.flat[i]!r}")


def rel_err_stats(a, b, scale=None) -> dict:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim == 2:
        d = np.linalg.norm(a - b, axis=1)
        s = np.linalg.norm(b, axis=1) if scale is None else scale
    else:
        d = np.abs(a - b)
        s = np.abs(b) if scale is None else scale
    r = d / np.maximum(s, 1e-30)
    return {"p50": float(np.quantile(r, 0.5)), "p99": float(np.quantile(r, 0.99)),
            "max": float(r.max())}


def check_grid_invariants(counts, starts, cell_idx, s2o, n: int) -> None:
    """Size-independent properties of the grid build (any N)."""
    counts = counts.astype(np.int64)
    starts = starts.astype(np.int64)
    assert counts.sum() == n
    assert np.array_equal(starts, np.cumsum(counts))
    # s2o and cell_idx are inverse permutations of [0, n)
    assert np.array_equal(np.sort(s2o[:n]), np.arange(n))
    assert np.array_equal(cell_idx[s2o[:n]], np.arange(n))
    # stable order: inside every cell, original indices ascend
    begins = starts - counts
    cell_of_slot = np.repeat(np.arange(len(counts)), counts)
    same_cell = cell_of_slot[1:] == cell_of_slot[:-1]
    assert (s2o[1:n][same_cell] > s2o[:n - 1][same_cell]).all()
    assert begins[0] == 0
