"""GPU parity of the batched Laplacian pyramid against the oracle.

All three launch forms (one persistent launch over a work-list of every level
of every image; one launch per level; the reference's per-image per-level
blur / subsample / difference launches) must give the oracle's pyramid bit for
bit (blur taps row-major with fused multiply-add; nearest-neighbour and linear
filtering mappings in FP32 with the contracted mapping), and the collapse must
restore the input (Restore, samples-public/5_Other/Gaussian_Laplacian_Pyramid).
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = [(257, 300), (300, 257), (513, 129), (97, 1001), (64, 64), (130, 66)]


def _plan(api, oracle, sizes, levels, boundary, seed):
    rng = np.random.default_rng(seed)
    imgs = [rng.random((h, w), dtype=np.float32) for (w, h) in sizes]
    plan = api.PyramidPlan([w for w, _ in sizes], [h for _, h in sizes], levels, oracle.binomial5(), boundary)
    for i, im in enumerate(imgs):
        plan.gauss(i, 0).copy_(torch.from_numpy(im).cuda())
    return plan, imgs


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_pyramid_bitexact(gpu, oracle, mode):
    levels = 6
    plan, imgs = _plan(gpu, oracle, SIZES, levels, oracle.MIRROR, 1)
    plan.decompose(mode)
    torch.cuda.synchronize()
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1)
        for l in range(levels):
            assert np.array_equal(plan.gauss(i, l).cpu().numpy(), g[l]), (mode, i, l)
            if l + 1 < levels:
                assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l]), (mode, i, l)
    plan.close()


def test_pyramid_persistent_many_images_and_collapse(gpu, oracle):
    """A longer work-list (24 images) through the persistent launch, then the
    collapse restores every input."""
    rng = np.random.default_rng(5)
    sizes = [(int(rng.integers(64, 600)), int(rng.integers(64, 600))) for _ in range(24)]
    levels = 6
    plan, imgs = _plan(gpu, oracle, sizes, levels, oracle.MIRROR, 2)
    plan.decompose(0)
    torch.cuda.synchronize()
    g0 = []
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1)
        assert np.array_equal(plan.gauss(i, levels - 1).cpu().numpy(), g[-1])
        assert np.array_equal(plan.lap(i, 0).cpu().numpy(), lap[0])
        g0.append(oracle.pyramid_collapse(g[-1], lap, contract=1)[0])
    plan.collapse()
    torch.cuda.synchronize()
    for i, im in enumerate(imgs):
        r = plan.gauss(i, 0).cpu().numpy()
        assert np.array_equal(r, g0[i])
        assert np.max(np.abs(r - im)) < 1e-5
    plan.close()


@pytest.mark.parametrize("boundary", [1, 2])
def test_pyramid_other_boundaries(gpu, oracle, boundary):
    levels = 5
    plan, imgs = _plan(gpu, oracle, SIZES[:3], levels, boundary, 3)
    plan.decompose(0)
    torch.cuda.synchronize()
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), boundary, contract=1)
        for l in range(levels - 1):
            assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l])
    plan.close()


def test_pyramid_status_clean(gpu):
    import ctypes as C

    from hipacc_gb300 import _lib as L

    st = C.c_int(-1)
    L.call("hgb_device_status", C.byref(st))
    assert st.value == 0


def test_pyramid_full_batch_all_modes(gpu, oracle):
    """The batching workload exactly as it is benchmarked: 64 FP32 images with
    w, h uniform in [257, 4096] (seed 4096), 8 levels, MIRROR.  Level 7 comes
    down to 2-3 pixels on some images (the repeated MIRROR reflection), and the
    persistent launch walks a work-list of every tile of every level.  Every
    G_l and L_l of every image must equal the oracle's in all three launch
    forms; outputs are poisoned with NaN first, so a tile that was never
    written fails."""
    from hipacc_gb300 import _lib as L

    rng = np.random.default_rng(4096)
    ws = rng.integers(257, 4097, 64)
    hs = rng.integers(257, 4097, 64)
    levels = 8
    assert min(int(ws.min()), int(hs.min())) >> (levels - 1) <= 3  # the tiny-level regime is exercised
    mask = oracle.binomial5()
    plans = [gpu.PyramidPlan(ws, hs, levels, mask, oracle.MIRROR) for _ in range(3)]
    imgs = []
    prng = np.random.default_rng(77)
    for i in range(64):
        im = prng.random((int(hs[i]), int(ws[i])), dtype=np.float32)
        imgs.append(im)
        d = torch.from_numpy(im).cuda()
        for p in plans:
            p.gauss(i, 0).copy_(d)
            for l in range(1, levels):
                p.gauss(i, l).fill_(float("nan"))
            for l in range(levels - 1):
                p.lap(i, l).fill_(float("nan"))
    for mode, p in enumerate(plans):
        p.decompose(mode)
    torch.cuda.synchronize()
    st = C.c_int(-1)
    L.call("hgb_device_status", C.byref(st))
    assert st.value == 0
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, mask, oracle.MIRROR, contract=1)
        gd = [torch.from_numpy(a).cuda() for a in g]
        ld = [torch.from_numpy(a).cuda() for a in lap]
        for mode, p in enumerate(plans):
            for l in range(levels):
                assert torch.equal(p.gauss(i, l), gd[l]), (mode, i, l)
                if l + 1 < levels:
                    assert torch.equal(p.lap(i, l), ld[l]), (mode, i, l)
    for p in plans:
        p.close()


@pytest.mark.parametrize("kind,level,mode", [(1, 0, 0), (1, 2, 0), (2, 1, 0), (2, 0, 1)])
def test_pyramid_bounded_waits_expire(gpu, oracle, kind, level, mode):
    """A wait that can never be satisfied runs out after a short poll limit:
    kind 1 withholds the completion of a level's tiles (the next level's
    inter-level waits run out), kind 2 issues no copy for a level's staged
    boxes (their barrier waits run out).  The launch ends by itself with
    HGB_ERR_TIMEOUT in the device status word, and the same plan then decomposes
    correctly once the test mode is off."""
    from hipacc_gb300 import _lib as L

    levels = 5
    plan, imgs = _plan(gpu, oracle, SIZES[:4], levels, oracle.MIRROR, 9)
    plan.wait_test(max_polls=2000, kind=kind, level=level)
    plan.decompose(mode)
    st = C.c_int(-1)
    L.call("hgb_device_status", C.byref(st))  # synchronises, reads and clears the word
    assert st.value == L.ERR_TIMEOUT
    plan.wait_test(0, 0, 0)
    plan.decompose(mode)
    L.call("hgb_device_status", C.byref(st))
    assert st.value == 0
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1)
        for l in range(levels - 1):
            assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l]), (i, l)
            assert np.array_equal(plan.gauss(i, l + 1).cpu().numpy(), g[l + 1]), (i, l)
    plan.close()


def test_pyramid_wait_test_arguments(gpu, oracle):
    from hipacc_gb300 import _lib as L

    plan, _ = _plan(gpu, oracle, SIZES[:1], 3, oracle.MIRROR, 1)
    lib = L.load()
    assert lib.hgb_pyramid_plan_wait_test(plan._h, -1, 0, 0) == L.ERR_INVALID
    assert lib.hgb_pyramid_plan_wait_test(plan._h, 10, 3, 0) == L.ERR_INVALID
    assert lib.hgb_pyramid_plan_wait_test(plan._h, 10, 1, 2) == L.ERR_INVALID  # the last level has no tiles
    assert lib.hgb_pyramid_plan_wait_test(None, 10, 1, 0) == L.ERR_INVALID
    plan.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_pyramid_every_tile_configuration(gpu, oracle, mode, tmp_path):
    """Every configuration the autotuner can choose for the fused launches
    (tile shape and threads; for the single launch also persistent claiming
    CTAs, one CTA per tile, or a cooperative grid sharing level 0 statically),
    forced through a loaded choice file, is bit-exact."""
    import json
    import math

    from hipacc_gb300 import _lib as L

    levels = 6
    plan, imgs = _plan(gpu, oracle, SIZES, levels, oracle.MIRROR, 12)
    px = sum(w * h for (w, h) in SIZES)
    key = "pyramid:m%d:n%d:l%d:px2^%d" % (mode, len(SIZES), levels, math.ceil(math.log2(px)))
    refs = [oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1) for im in imgs]
    for k in range(12 if mode == 0 else 4):
        f = tmp_path / "choice.json"
        f.write_text(json.dumps({key: [k, 0.0]}))
        L.call("hgb_autotune_clear")
        L.call("hgb_autotune_load", str(f).encode())
        for i in range(len(SIZES)):
            for l in range(1, levels):
                plan.gauss(i, l).fill_(float("nan"))
        plan.decompose(mode)
        torch.cuda.synchronize()
        for i, (g, lap) in enumerate(refs):
            for l in range(levels):
                assert np.array_equal(plan.gauss(i, l).cpu().numpy(), g[l]), (k, i, l)
                if l + 1 < levels:
                    assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l]), (k, i, l)
    L.call("hgb_autotune_clear")
    st = C.c_int(-1)
    L.call("hgb_device_status", C.byref(st))
    assert st.value == 0
    plan.close()


def test_pyramid_autotuner_picks_and_keeps_a_choice(gpu, oracle, tmp_path):
    """With autotuning on, the first decomposition times the configurations
    and stores one choice per (launch form, batch shape); results stay exact."""
    from hipacc_gb300 import _lib as L

    L.call("hgb_autotune_clear")
    gpu.autotune(True)
    try:
        plan, imgs = _plan(gpu, oracle, SIZES[:3], 5, oracle.MIRROR, 13)
        n0 = L.load().hgb_autotune_count()
        plan.decompose(0)
        plan.decompose(1)
        torch.cuda.synchronize()
        assert L.load().hgb_autotune_count() == n0 + 2
        for i, im in enumerate(imgs):
            g, lap = oracle.pyramid_decompose(im, 5, oracle.binomial5(), oracle.MIRROR, contract=1)
            assert np.array_equal(plan.lap(i, 0).cpu().numpy(), lap[0])
            assert np.array_equal(plan.gauss(i, 4).cpu().numpy(), g[4])
        f = tmp_path / "tuned.json"
        L.call("hgb_autotune_save", str(f).encode())
        assert "pyramid:m0" in f.read_text() and "pyramid:m1" in f.read_text()
        plan.close()
    finally:
        gpu.autotune(False)
        L.call("hgb_autotune_clear")


@pytest.mark.parametrize("k", [0, 4, 8])
def test_pyramid_single_launch_in_a_graph(gpu, oracle, k, tmp_path):
    """Each form of the single launch (persistent claiming, one CTA per tile,
    cooperative static level 0) is recorded into a CUDA graph and replayed."""
    import json
    import math

    from hipacc_gb300 import _lib as L

    levels = 6
    plan, imgs = _plan(gpu, oracle, SIZES, levels, oracle.MIRROR, 14)
    px = sum(w * h for (w, h) in SIZES)
    key = "pyramid:m0:n%d:l%d:px2^%d" % (len(SIZES), levels, math.ceil(math.log2(px)))
    f = tmp_path / "choice.json"
    f.write_text(json.dumps({key: [k, 0.0]}))
    L.call("hgb_autotune_clear")
    L.call("hgb_autotune_load", str(f).encode())
    try:
        s = torch.cuda.Stream()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            plan.decompose(0, stream=s)
        for i in range(len(SIZES)):
            for l in range(levels - 1):
                plan.lap(i, l).fill_(float("nan"))
        torch.cuda.synchronize()
        g.replay()
        g.replay()
        torch.cuda.synchronize()
        for i, im in enumerate(imgs):
            _, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1)
            for l in range(levels - 1):
                assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l]), (k, i, l)
    finally:
        L.call("hgb_autotune_clear")
        plan.close()


def test_pyramid_trace_records(gpu, oracle, tmp_path):
    """The single launch's per-CTA trace (hgb_pyramid_plan_trace) in each form:
    the traced launch is still bit-exact, every tile is counted once, and every
    record is well formed (end after start, parts within the CTA's lifetime)."""
    import json
    import math

    from hipacc_gb300 import _lib as L

    levels = 6
    plan, imgs = _plan(gpu, oracle, SIZES, levels, oracle.MIRROR, 13)
    px = sum(w * h for (w, h) in SIZES)
    key = "pyramid:m0:n%d:l%d:px2^%d" % (len(SIZES), levels, math.ceil(math.log2(px)))
    refs = [oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1) for im in imgs]
    buf = torch.zeros(8 * 20000, dtype=torch.int64, device="cuda")
    counts = []
    for single in (0, 1, 2):
        f = tmp_path / "choice.json"
        f.write_text(json.dumps({key: [single * 4, 0.0]}))
        L.call("hgb_autotune_clear")
        L.call("hgb_autotune_load", str(f).encode())
        buf.zero_()
        plan.trace(buf)
        plan.decompose(0)
        torch.cuda.synchronize()
        plan.trace(None)
        r = buf.view(-1, 8).cpu().numpy()
        r = r[r[:, 1] > 0]
        assert len(r) > 0
        assert np.all(r[:, 1] >= r[:, 0]) and np.all(r[:, 3] >= r[:, 2])
        life = r[:, 3] - r[:, 2]
        assert np.all(r[:, 4] + r[:, 5] + r[:, 6] <= life)
        ntiles = int((r[:, 7] & 0xffffffff).sum())
        counts.append(ntiles)
        for i, (g, lap) in enumerate(refs):
            for l in range(levels):
                assert np.array_equal(plan.gauss(i, l).cpu().numpy(), g[l]), (single, i, l)
                if l + 1 < levels:
                    assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l]), (single, i, l)
    # the same work-list in every form: each tile taken exactly once
    assert counts[0] > 0 and counts[0] == counts[1] == counts[2], counts
    L.call("hgb_autotune_clear")
    plan.close()
