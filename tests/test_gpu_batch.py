"""Batched frames (drv_batch_*): scenes of different sizes captured into one
graph over several streams give each scene the frame its own drv_frame
gives; completion times are ordered within the batch total."""
import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, batch, pipeline, surrogate

pytestmark = pytest.mark.gpu


def _small_specs(visibility, precision):
    base = pipeline.WORKLOADS["c1_small"]
    specs = []
    for i, (res, vox, cav) in enumerate([(128, 64, 32), (192, 64, 32), (256, 128, 32), (160, 128, 64)]):
        w = pipeline.scaled(base, name=f"b{i}", width=res, height=res, voxel_res=vox, cav_res=cav, n_cascades=2,
                            cascade_world_size0=1.0, sh_order=2, max_caches=16384, visibility=visibility,
                            precision=precision)
        specs.append((w, 40 + i))
    return specs


@pytest.mark.parametrize("visibility,precision", [(abi.VISIBILITY_CONE, abi.PRECISION_FP32),
                                                  (abi.VISIBILITY_SURROGATE, abi.PRECISION_BF16)],
                         ids=["cone_fp32", "surrogate_bf16"])
@pytest.mark.parametrize("streams", [1, 3])
def test_batch_equals_each_scenes_frame(visibility, precision, streams, cuda, lib):
    import torch
    scenes = batch.make_scenes(_small_specs(visibility, precision), threshold=0.5, params=surrogate.init_params(3))
    direct = [s.pipe.out.clone() for s in scenes]  # make_scenes ran one drv_frame per scene
    for s in scenes:
        s.pipe.out.zero_()
    torch.cuda.synchronize()  # the batch's streams do not wait for the default stream
    b = batch.Batch(scenes, streams)
    total, per = b.run()
    torch.cuda.synchronize()
    for s, d in zip(scenes, direct):
        assert torch.equal(s.pipe.out, d)
    assert total > 0 and np.all(per > 0) and np.all(per <= total + 1e-3)
    b.close()
    for s in scenes:
        s.pipe.close()


def test_batch_rejects_bad_arguments(cuda, lib):
    import ctypes as C
    h = C.c_void_p()
    assert lib.drv_batch_create(None, 1, 1, None, C.byref(h)) == abi.ERR_INVALID_ARG
    tab = (abi.DrvBatchScene * 1)()
    assert lib.drv_batch_create(tab, 1, 1, None, C.byref(h)) == abi.ERR_INVALID_ARG  # null context
    assert lib.drv_batch_launch(None, None) == abi.ERR_INVALID_ARG
