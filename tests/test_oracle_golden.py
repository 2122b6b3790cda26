"""The oracle still produces the committed golden frame (tests/golden,
written by make_golden.py): a change to the oracle that moves any stage's
output shows up here."""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).with_name("golden")


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN / "tiny_frame.npz"))


def test_oracle_reproduces_the_golden_frame(golden, oracle):
    sys.path.insert(0, str(GOLDEN))
    import make_golden
    now = make_golden.frame()
    assert set(now) == set(golden)
    for k in ("normal16", "rsm_normal16", "voxel_bits", "cache_count"):
        assert np.array_equal(now[k], golden[k]), k
    for k in ("depth", "albedo", "rsm_flux", "rsm_dls", "vpls", "cones", "mips", "cache_positions", "cache_sh",
              "radiance"):
        assert np.allclose(now[k], golden[k], rtol=1e-12, atol=0), k


def test_golden_frame_is_not_trivial(golden):
    assert int(golden["cache_count"]) > 100
    assert np.count_nonzero(golden["radiance"]) > 0.5 * golden["radiance"].size
    assert 0 < golden["voxel_bits"].view(np.uint8).sum()
