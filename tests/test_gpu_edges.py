"""Edge cases of the path, each through every stage: a frame with no geometry
(no caches at all), lights without flux (no contributing pair), resolutions
that are not multiples of the 16 x 16 tiles, a tiny RSM, and the largest
number of lights a frame takes (DRV_MAX_LIGHTS). Checked against the exact
answer or the FP64 oracle frame from the same inputs."""
import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline
from test_gpu_parity import Run, oracle_frame, rel_l2

pytestmark = pytest.mark.gpu

C1 = pipeline.WORKLOADS["c1_small"]


def _after_inputs(w, edit, **knobs):
    """Pipeline with ray-cast inputs, `edit(pipe)` applied to them (on torch's
    stream, synchronised both ways), then every stage."""
    import torch
    p = pipeline.Pipeline(pipeline.host_frame(w))
    if knobs:
        p.set_tuning(**knobs)
    p.raycast_inputs()
    p.sync()
    edit(p)
    torch.cuda.synchronize()
    p.prepare_and_extract()
    p.voxelize()
    p.allocate()
    p.light()
    p.apply()
    p.sync()
    return p


@pytest.mark.parametrize("path", [abi.LIGHT_PATH_SPLIT, abi.LIGHT_PATH_SINGLE], ids=["split", "single"])
def test_frame_without_geometry_allocates_nothing_and_shades_zero(path, cuda, lib):
    """Every depth 0 (cacheApply.frag:304-307 discards, cacheGather.comp
    allocates nothing): no cache, an empty light stage, zero radiance
    written over whatever the target held; drv_frame the same."""
    def edit(p):
        p.depth.zero_()
        p.out.fill_(7.0)
    p = _after_inputs(C1, edit, light_path=path)
    assert p.cache_count() == 0
    assert np.all(p.out.cpu().numpy() == 0)
    p.out.fill_(7.0)
    p.frame()
    p.sync()
    assert p.cache_count() == 0
    assert np.all(p.out.cpu().numpy() == 0)
    p.close()


def test_lights_without_flux_give_no_pairs_and_zero_radiance(cuda, lib):
    """Black RSM flux: no VPL can contribute, so the cull lists no pair, the
    caches keep zero SH and every pixel's radiance is exactly 0."""
    def edit(p):
        for f in p.rsm_flux:
            f.zero_()
    p = _after_inputs(C1, edit, light_path=abi.LIGHT_PATH_SPLIT)
    assert p.cache_count() > 0
    assert p.light_pairs() == 0
    _, sh = p.read_entries_decoded(p.cache_count())
    assert np.all(sh == 0)
    assert np.all(p.out.cpu().numpy() == 0)
    p.close()


@pytest.mark.parametrize("w", [
    pipeline.scaled(C1, name="c1_odd", width=257, height=131),
    pipeline.scaled(C1, name="c1_tiny_rsm", rsm_read_lod=3),
    pipeline.scaled(C1, name="c1_tiny_rsm_blocks", rsm_read_lod=3, shadow_lod=1),
    pipeline.scaled(C1, name="c1_max_lights", n_lights=16, rsm_read_lod=2, max_caches=8192),
], ids=["odd_257x131", "rsm_4x4", "rsm_4x4_blocks_of_4", "16_lights"])
def test_edge_shapes_match_fp64(w, lib, oracle, cuda):
    """Ragged image edges (257 x 131: partial tiles in x and y), an RSM read
    at 4 x 4 (16 VPLs; with shadow blocks of 4: 4 cones), and 16 spot lights
    accumulating into every entry: allocation bit-exact, the whole frame
    within the 1% relative L2 of the FP64 oracle frame."""
    r = Run(w, oracle)
    st, atlas, pos, count = oracle.allocate_caches(r.hf.config, r.hf.volume, r.hf.frame, r.depth)
    assert r.count == count
    assert np.array_equal(r.atlas != 0, atlas != 0)
    ref = oracle_frame(r, oracle)
    err = rel_l2(r.out, ref)
    print("%s: %d caches, frame rel-L2 %.2e" % (w.name, r.count, err))
    assert np.abs(ref).max() > 0
    assert err < 1e-2, err
    r.pipe.close()
