"""The shipped surrogate checkpoints (CPU): each loads with the parameter
count of the MLP, names a feature set the library knows, records its
training run and its held-out evaluation, and the default one is cone4."""
import json

import numpy as np

from dynamicradiancevolume_gb300 import abi, surrogate


def test_shipped_checkpoints_are_complete():
    paths = sorted(surrogate.DEFAULT_WEIGHTS.parent.glob("*.json"))
    assert len(paths) >= 3
    for p in paths:
        stem = p.with_suffix("")
        params = surrogate.load_params(stem)
        assert params.shape == (abi.SURROGATE_PARAMS,) and np.isfinite(params).all()
        features = surrogate.load_features(stem)
        assert features in abi.SURROGATE_FEATURE_NAMES
        header = json.loads(p.read_text())
        assert header["trained_on"]["scene_seeds"][1] < 1000 <= header["held_out"]["scene_seeds"][0]
        assert 0.0 < header["held_out"]["mae"] < 1.0
    assert surrogate.load_features(surrogate.DEFAULT_WEIGHTS) == "cone4"
