"""Brute-force RSM gather (Renderer::ApplyRSMsBruteForce, bruteforcersm.frag)
against the FP64 oracle on the GPU's own G-buffer and VPLs, with the diffuse
and with the reference BRDF; and the interpolation error of the cache path
measured against it (both unshadowed)."""
import numpy as np
import pytest

from dynamicradiancevolume_gb300 import abi, pipeline
from test_gpu_parity import REDUCED, Run, oracle_frame, rel_l2

pytestmark = pytest.mark.gpu

NOSHADOW = pipeline.scaled(pipeline.WORKLOADS["c1_small"], name="c1_noshadow", indirect_shadow=0, sh_order=2)


@pytest.fixture(scope="module")
def ns(lib, oracle, cuda):
    return Run(NOSHADOW, oracle, seed=17)


def test_bruteforce_matches_fp64(ns, oracle):
    out = ns.pipe.bruteforce().cpu().numpy()
    ref = oracle.bruteforce_rsm(ns.hf.frame, ns.depth, ns.n16, ns.albedo, ns.gpu_vpls_f64())
    assert np.count_nonzero(ref) > 0.5 * ref.size
    assert rel_l2(out, ref) < 1e-5


def test_bruteforce_reference_brdf_matches_fp64(ns, oracle):
    torch = ns.torch
    g = torch.Generator().manual_seed(3)
    H, W = ns.depth.shape
    rm = torch.stack([torch.rand(H, W, generator=g) * 0.8 + 0.2, torch.rand(H, W, generator=g)], -1)
    out = ns.pipe.bruteforce(rough_metal=rm.cuda()).cpu().numpy()
    ref = oracle.bruteforce_rsm(ns.hf.frame, ns.depth, ns.n16, ns.albedo, ns.gpu_vpls_f64(),
                                rough_metal=rm.numpy())
    assert rel_l2(out, ref) < 1e-4


def test_cache_interpolation_error_against_bruteforce(ns, oracle):
    # Unshadowed cache path vs the per-pixel ground truth on the same inputs:
    # the error the cache volume's interpolation introduces (a property of
    # the method, reported; bounded here only to catch a broken path).
    brute = ns.pipe.bruteforce().cpu().numpy()
    err = rel_l2(ns.out, brute)
    print(f"cache path vs brute force (unshadowed, {NOSHADOW.name}): rel-L2 {err:.4f}")
    assert err < 0.5
