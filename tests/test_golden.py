"""Golden fixtures of the SPH step, generated from the reference's own WGSL
step shaders (translated mechanically to C++; tests/golden/make_golden.py).

CPU: the oracle restatement reproduces every fixture bit for bit.
GPU: the sm_103a library through its C ABI reproduces every fixture bit for
bit (digests over canonicalised buffers: -0 -> +0, NaN -> one NaN)."""
import json
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent / "golden"
MANIFEST = json.loads((HERE / "manifest.json").read_text())
CASES = list(MANIFEST["cases"])


@pytest.fixture(scope="module")
def golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", HERE / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod, np.load(HERE / "step_fixtures.npz")


def _check(out, name, golden):
    mod, arrays = golden
    entry = MANIFEST["cases"][name]
    assert len(out["particles"]) == entry["n"]
    assert list(out["accum"]) == entry["accum"], "rigid-body accumulator"
    for k, want in entry["digests"].items():
        got = mod.digest(out[k])
        if got != want:
            key = f"{name}/{k}"
            if key in arrays:
                a = mod.canon(out[k])
                b = arrays[key]
                bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
                raise AssertionError(f"{name}: {k} differs at {bad[:3].tolist()}")
            raise AssertionError(f"{name}: digest of {k} differs from the reference fixture")
    if f"{name}/particles_sample" in arrays:
        idx = np.arange(0, entry["n"], mod.SAMPLE_STRIDE)
        np.testing.assert_array_equal(mod.canon(out["particles"][idx]),
                                      arrays[f"{name}/particles_sample"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(oracle_mod, golden, name):
    mod, _ = golden

    def make(sc, sdf):
        return oracle_mod.oracle_for_scene(sc, sdf=sdf)

    _check(mod.run_case(name, make), name, golden)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_fixture(fslib, golden, name):
    from helpers import gpu_sim_for_scene
    mod, _ = golden
    _check(mod.run_case(name, lambda sc, sdf: gpu_sim_for_scene(sc, sdf=sdf)), name, golden)
