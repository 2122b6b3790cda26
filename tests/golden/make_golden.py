"""Writes tests/golden/tiny_frame.npz: one tiny seeded frame through the FP64
oracle, inputs and every stage's output, so that later oracle changes are
caught (test_oracle_golden.py) and the GPU path is checked on exactly these
inputs (test_gpu_golden.py). The reference cannot run on these machines (its
shaders need an OpenGL 4.5 context), so the fixtures are the oracle's.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle_py as O  # noqa: E402
from dynamicradiancevolume_gb300 import pipeline  # noqa: E402

# 48x32 pixels, 8 boxes, 32^3 voxels, one light with a 16^2 RSM (256 VPLs),
# one 16^3 cascade, SH2, 8 cone steps.
TINY = pipeline.scaled(pipeline.WORKLOADS["c1_small"], name="golden_tiny", width=48, height=32, n_boxes=8,
                       voxel_res=32, rsm_resolution=16, cav_res=16, sh_order=2, max_cone_steps=8, max_caches=4096)
SEED = 5


def frame():
    w = TINY
    hf = pipeline.host_frame(w, SEED)
    depth, n16, n32, alb = O.raycast_gbuffer(hf.boxes, hf.scene.n_boxes, hf.frame, hf.camera, w.width, w.height)
    flux, rn, dls = O.raycast_rsm(hf.boxes, hf.scene.n_boxes, hf.lights[0])
    chain = O.rsm_chain(flux, rn, dls, w.rsm_read_lod + w.shadow_lod)
    vpls, cones = O.extract_vpls(hf.lights[0], *chain[w.rsm_read_lod], chain[w.rsm_read_lod + w.shadow_lod][2])
    bits = O.voxelize(hf.boxes, hf.scene.n_boxes, hf.volume, w.voxel_res)
    mips = O.build_mips(w.voxel_res, bits)
    st, atlas, pos, count = O.allocate_caches(hf.config, hf.volume, hf.frame, depth)
    sh = O.light_caches(hf.config, hf.volume, pos, hf.lights, [vpls], [cones], bits, mips, n_threads=1)
    out = O.apply(hf.config, hf.volume, hf.frame, depth, n16, 0, alb, atlas, sh, n_threads=1)
    order = np.lexsort(pos.T[::-1])  # caches by position (allocation order is atomic order on the GPU)
    return dict(depth=depth, normal16=n16, albedo=alb, rsm_flux=flux, rsm_normal16=rn, rsm_dls=dls, vpls=vpls,
                cones=cones, voxel_bits=bits, mips=mips, cache_positions=pos[order], cache_sh=sh[order],
                cache_count=np.array(count), radiance=out)


if __name__ == "__main__":
    np.savez_compressed(Path(__file__).with_name("tiny_frame.npz"), **frame())
    print("wrote", Path(__file__).with_name("tiny_frame.npz"))
