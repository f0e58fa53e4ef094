"""GPU parity of the integer pipeline: Sobel magnitude with fused sum / max,
RGBA -> gray, and standalone reductions.  Bar: bit-exact."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sobel(api, img, b=3, const=0, mx=None, my=None, batch=False):
    t = torch.from_numpy(img).cuda()
    out = torch.zeros_like(t)
    s = torch.zeros(1, dtype=torch.int64, device="cuda")
    m = torch.zeros(1, dtype=torch.int32, device="cuda")
    kw = {}
    if mx is not None:
        kw = dict(mask_x=mx, mask_y=my)
    api.sobel_mag(t, out, boundary=b, const=const, sum_out=s, max_out=m, **kw)
    torch.cuda.synchronize()
    return out.cpu().numpy(), int(s.item()), int(m.item())


@pytest.mark.parametrize("b", [1, 2, 3, 4])
@pytest.mark.parametrize("hw", [(64, 128), (21, 37), (200, 301), (1, 1), (2, 2), (3, 1000), (129, 129)])
def test_sobel_bitexact(gpu, oracle, b, hw):
    rng = np.random.default_rng(hash((b, hw)) % 2**32)
    img = rng.integers(0, 256, hw, dtype=np.uint8)
    out, s, m = _sobel(gpu, img, b=b, const=17)
    ref = oracle.sobel_mag(img, boundary=b, const=17)
    assert np.array_equal(out, ref)
    assert s == oracle.reduce_sum_u8(ref) and m == oracle.reduce_max_u8(ref)


@pytest.mark.parametrize("b", [1, 2, 3, 4])
@pytest.mark.parametrize("hw", [(129, 129), (200, 301), (1, 1), (3, 1000), (1001, 333), (35, 4097), (257, 128)])
def test_sobel_pitched_tma_path(gpu, oracle, b, hw):
    """Rows padded to a multiple of 16 bytes make any width TMA-legal: ragged
    right and bottom tiles and one-row images through the staged fast path,
    one image and a batch of three."""
    rng = np.random.default_rng(hash(("p", b, hw)) % 2**32)
    h, w = hw
    wp = (w + 15) // 16 * 16 + 16
    imgs = rng.integers(0, 256, (3, h, w), dtype=np.uint8)
    dev = torch.zeros((3, h, wp), dtype=torch.uint8, device="cuda")
    dev[:, :, :w] = torch.from_numpy(imgs).cuda()
    out = torch.full((3, h, wp), 7, dtype=torch.uint8, device="cuda")
    for batch in (False, True):
        s = torch.zeros(1, dtype=torch.int64, device="cuda")
        m = torch.zeros(1, dtype=torch.int32, device="cuda")
        src = dev[:, :, :w] if batch else dev[0, :, :w]
        dst = out[:, :, :w] if batch else out[0, :, :w]
        gpu.sobel_mag(src, dst, boundary=b, const=17, sum_out=s, max_out=m)
        torch.cuda.synchronize()
        refs = [oracle.sobel_mag(imgs[i], boundary=b, const=17) for i in range(3 if batch else 1)]
        got = out.cpu().numpy()
        for i, ref in enumerate(refs):
            assert np.array_equal(got[i, :, :w], ref), (batch, i)
            assert np.all(got[i, :, w:] == 7)  # nothing written past the width
        assert s.item() == sum(int(r.astype(np.uint64).sum()) for r in refs)
        assert m.item() == max(int(r.max()) for r in refs)


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4])
def test_sobel_every_tile_configuration(gpu, oracle, cfg, tmp_path):
    """Each configuration the autotuner can choose for the staged Sobel (rows
    per warp; one CTA per tile, or a few CTAs per SM claiming tiles), forced
    through a loaded choice file, is bit-exact: ragged tiles, warps whose rows
    lie below the image, every boundary mode, low-contrast images whose
    maximum is below 255, a batch, and calls with and without the fused
    sum / max one after the other (the claim counter returns to zero)."""
    import json

    from hipacc_gb300 import _lib as L

    rng = np.random.default_rng(40 + cfg)
    cases = [((777, 1001), 3, 256, 1), ((512, 512), 3, 256, 1), ((4096, 4096), 3, 256, 1),
             ((100, 300), 1, 256, 1), ((33, 129), 2, 256, 1), ((1, 64), 4, 256, 1), ((130, 17), 3, 256, 1),
             ((300, 700), 3, 9, 1), ((257, 390), 4, 256, 3), ((96, 160), 2, 5, 2)]
    for (h, w), bnd, hi, nb in cases:
        imgs = rng.integers(0, hi, (nb, h, w), dtype=np.uint8)
        wp = (w + 15) // 16 * 16
        dev = torch.zeros((nb, h, wp), dtype=torch.uint8, device="cuda")
        dev[:, :, :w] = torch.from_numpy(imgs).cuda()
        out = torch.zeros((nb, h, wp), dtype=torch.uint8, device="cuda")
        key = "sobel3:%dx%dx%d" % (1 << w.bit_length(), 1 << h.bit_length(), nb)
        f = tmp_path / "choice.json"
        f.write_text(json.dumps({key: [cfg, 0.0]}))
        L.call("hgb_autotune_clear")
        L.call("hgb_autotune_load", str(f).encode())
        s = torch.zeros(1, dtype=torch.int64, device="cuda")
        m = torch.zeros(1, dtype=torch.int32, device="cuda")
        src, dst = (dev[:, :, :w], out[:, :, :w]) if nb > 1 else (dev[0, :, :w], out[0, :, :w])
        gpu.sobel_mag(src, dst, boundary=bnd, const=17)  # no sum / max
        torch.cuda.synchronize()
        refs = [oracle.sobel_mag(imgs[i], boundary=bnd, const=17) for i in range(nb)]
        got = out.cpu().numpy()
        for i, ref in enumerate(refs):
            assert np.array_equal(got[i, :, :w], ref), (h, w, bnd, i)
        out.zero_()
        gpu.sobel_mag(src, dst, boundary=bnd, const=17, sum_out=s, max_out=m)
        torch.cuda.synchronize()
        L.call("hgb_autotune_clear")
        got = out.cpu().numpy()
        for i, ref in enumerate(refs):
            assert np.array_equal(got[i, :, :w], ref), (h, w, bnd, i)
        assert s.item() == sum(int(r.astype(np.uint64).sum()) for r in refs), (h, w)
        assert m.item() == max(int(r.max()) for r in refs), (h, w)
    import ctypes as C

    status = C.c_int(-1)
    L.call("hgb_device_status", C.byref(status))
    assert status.value == L.OK


def test_sobel_4096_mirror(gpu, oracle):
    """The 4096x4096 u8 Sobel with MIRROR and the u64 sum / u8 max."""
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (4096, 4096), dtype=np.uint8)
    out, s, m = _sobel(gpu, img, b=3)
    ref = oracle.sobel_mag(img, boundary=3)
    assert np.array_equal(out, ref)
    assert s == oracle.reduce_sum_u8(ref, nthreads=8) == int(ref.astype(np.uint64).sum())
    assert m == oracle.reduce_max_u8(ref)


@pytest.mark.parametrize("size", [3, 5, 7])
def test_sobel_generic_masks(gpu, oracle, size):
    """Sample masks of size 5 and 7 (and a non-standard 3x3) take the general kernel."""
    rng = np.random.default_rng(size)
    mx = rng.integers(-3, 4, (size, size)).astype(np.int32)
    my = rng.integers(-3, 4, (size, size)).astype(np.int32)
    img = rng.integers(0, 256, (45, 70), dtype=np.uint8)
    for b in (1, 3, 4):
        out, s, m = _sobel(gpu, img, b=b, const=9, mx=mx, my=my)
        ref = oracle.sobel_mag(img, mask_x=mx, mask_y=my, boundary=b, const=9)
        assert np.array_equal(out, ref)
        assert s == int(ref.astype(np.uint64).sum()) and m == int(ref.max())


def test_sobel_repeated_calls_reset_ticket(gpu, oracle):
    rng = np.random.default_rng(3)
    for i in range(4):
        img = rng.integers(0, 256, (300 + i, 500 - i), dtype=np.uint8)
        out, s, m = _sobel(gpu, img)
        assert s == int(oracle.sobel_mag(img, boundary=3).astype(np.uint64).sum())


@pytest.mark.parametrize("hw", [(4096, 4096), (17, 33), (1, 5), (64, 1), (1000, 999), (5, 8192), (3, 1367)])
def test_gray_bitexact(gpu, oracle, hw):
    # dense images of at least one 4096-pixel unit take the bulk-copy pipeline
    # (whole units + a ragged tail); smaller ones the vector kernel
    rng = np.random.default_rng(hw[0])
    rgba = rng.integers(0, 256, hw + (4,), dtype=np.uint8)
    t = torch.from_numpy(rgba).cuda()
    out = gpu.gray(t)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.rgba_to_gray(rgba))


def test_gray_pitched_and_weights(gpu, oracle):
    rng = np.random.default_rng(4)
    rgba = rng.integers(0, 256, (40, 50, 4), dtype=np.uint8)
    big = torch.zeros((40, 64, 4), dtype=torch.uint8, device="cuda")
    big[:, :50] = torch.from_numpy(rgba).cuda()
    out_big = torch.zeros((40, 80), dtype=torch.uint8, device="cuda")
    gpu.gray(big[:, :50], out_big[:, :50], weights=(300, 500, 100), shift=10)
    assert np.array_equal(out_big[:, :50].cpu().numpy(), oracle.rgba_to_gray(rgba, (300, 500, 100), 10))


@pytest.mark.parametrize("dtype,np_dt", [(torch.uint8, np.uint8), (torch.int16, np.int16), (torch.int32, np.int32)])
def test_reduce_integer(gpu, dtype, np_dt):
    rng = np.random.default_rng(5)
    info = np.iinfo(np_dt)
    a = rng.integers(max(info.min, -1000), min(info.max, 1000) + 1, (123, 457)).astype(np_dt)
    t = torch.from_numpy(a).cuda()
    assert gpu.reduce(t, 0) == int(a.astype(np.int64).sum())
    assert gpu.reduce(t, 1) == int(a.min())
    assert gpu.reduce(t, 2) == int(a.max())
    win = (13, 7, 100, 50)
    sub = a[7:57, 13:113]
    assert gpu.reduce(t, 0, win=win) == int(sub.astype(np.int64).sum())


def test_reduce_float_sum_accuracy(gpu, oracle):
    """Kahan partials + FP64 combine: far closer to the exact sum than the
    reference's FP32 fold (REDUCTION_CPU_2D)."""
    rng = np.random.default_rng(6)
    a = rng.random((4096, 4096), dtype=np.float32)
    t = torch.from_numpy(a).cuda()
    exact = oracle.reduce_f32_exact(a, 0)
    got = gpu.reduce(t, 0)
    assert abs(got - exact) / exact < 1e-9
    ref_fp32 = oracle.reduce_f32(a, 0, 8)
    assert abs(got - exact) <= abs(ref_fp32 - exact)
    assert gpu.reduce(t, 1) == float(a.min()) and gpu.reduce(t, 2) == float(a.max())
    assert gpu.reduce(t, 0) == got  # deterministic


def test_reduce_half_and_double(gpu):
    rng = np.random.default_rng(7)
    a = rng.random((300, 301))
    t = torch.from_numpy(a).cuda()
    assert abs(gpu.reduce(t, 0) - a.sum()) < 1e-9
    h = torch.from_numpy(a.astype(np.float32)).to(torch.bfloat16).cuda()
    assert abs(gpu.reduce(h, 0) - h.double().sum().item()) < 1e-6 * h.double().sum().item()


@pytest.mark.parametrize("hw", [(1, 1), (2, 3), (33, 17), (34, 129), (70, 300), (127, 161)])
@pytest.mark.parametrize("b", [1, 2, 3, 4])
def test_sobel_tma_pitched(gpu, oracle, hw, b):
    """Rows padded to a 16-byte pitch so the TMA path runs even on tiny and
    ragged images (box larger than the image, every tile a border tile)."""
    h, w = hw
    rng = np.random.default_rng(h * 1000 + w + b)
    img = rng.integers(0, 256, hw, dtype=np.uint8)
    pw = (w + 15) // 16 * 16 + 16
    src = torch.zeros((h, pw), dtype=torch.uint8, device="cuda")
    src[:, :w] = torch.from_numpy(img).cuda()
    dst = torch.zeros((h, pw), dtype=torch.uint8, device="cuda")
    s = torch.zeros(1, dtype=torch.int64, device="cuda")
    m = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu.sobel_mag(src[:, :w], dst[:, :w], boundary=b, const=200, sum_out=s, max_out=m)
    ref = oracle.sobel_mag(img, boundary=b, const=200)
    assert np.array_equal(dst[:, :w].cpu().numpy(), ref)
    assert int(dst[:, w:].sum().item()) == 0  # nothing written past the row
    assert int(s.item()) == int(ref.astype(np.uint64).sum()) and int(m.item()) == int(ref.max())


def test_sobel_batch_tma(gpu, oracle):
    """A batch of three images in one launch (one CTA per tile of every image);
    the fused sum / max cover the whole batch."""
    rng = np.random.default_rng(12)
    imgs = rng.integers(0, 256, (3, 200, 256), dtype=np.uint8)
    t = torch.from_numpy(imgs).cuda()
    out = torch.empty_like(t)
    s = torch.zeros(1, dtype=torch.int64, device="cuda")
    m = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu.sobel_mag(t, out, boundary=3, sum_out=s, max_out=m)
    refs = [oracle.sobel_mag(imgs[i], boundary=3) for i in range(3)]
    for i in range(3):
        assert np.array_equal(out[i].cpu().numpy(), refs[i])
    assert int(s.item()) == sum(int(r.astype(np.uint64).sum()) for r in refs)
    assert int(m.item()) == max(int(r.max()) for r in refs)


def test_device_status_clean(gpu):
    """No kernel recorded a bounded-wait timeout during the run."""
    import ctypes as C

    from hipacc_gb300 import _lib as L

    st = C.c_int(-1)
    L.call("hgb_device_status", C.byref(st))
    assert st.value == 0
