"""The CPU oracle against the committed golden fixtures (tests/golden/, made by make_golden.py):
the oracle must keep producing the frozen vis-buffers, colours, Hi-Z texels, cull bitmaps and
decoder gradients on the fixed seeded scenes."""
import os

import numpy as np
import pytest

from tests.golden import make_golden as G

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


@pytest.fixture(scope="module")
def O():
    from oracle import oracle as O
    O.lib()
    O.set_approx_mode(0)
    return O


@pytest.mark.parametrize("name", ["raster_grid", "raster_inside", "resolve_volume", "alpha_debug"])
def test_oracle_matches_golden(O, name):
    gold = load(name)
    out = G.MAKERS[name](O)
    assert out["scene_hash"] == str(gold["scene_hash"]), "the scene generator changed: regenerate the fixtures"
    for k, v in out.items():
        if k == "scene_hash":
            continue
        assert np.array_equal(np.asarray(v), gold[k]), f"{name}.{k} differs from the golden fixture"


def test_neural_oracle_matches_golden():
    gold = load("neural_fwd_bwd")
    out = G.make_neural(None)
    for k in ("y", "param_grad", "dx0"):
        assert np.allclose(out[k], gold[k], rtol=1e-12, atol=1e-15), k
    assert abs(float(out["loss"]) - float(gold["loss"])) <= 1e-12 * float(gold["loss"])
