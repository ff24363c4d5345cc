"""Parity of the preprocessing kernels (generator, mip, bricker, empty flags)
with the oracle, through the C ABI.  Integer data: bit-exact."""
import numpy as np
import pytest

import scenario

pytestmark = pytest.mark.gpu


def to_np(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("size,bpc,ch", [((37, 29, 23), 1, 1), ((64, 48, 40), 2, 1), ((40, 32, 24), 1, 2)])
def test_generator_matches_oracle(gc, orc, torch_cuda, size, bpc, ch):
    g = scenario.gpu_volume(gc, torch_cuda, size, bpc, 5, 6, channels=ch)
    o = scenario.orc_volume(orc, size, bpc, 5, 6, channels=ch)
    assert np.array_equal(to_np(g), o.reshape(-1).view(np.uint8))


MIP_CASES = [
    ((64, 48, 32), 1, 1), ((64, 48, 32), 2, 1), ((64, 48, 32), 4, 1), ((64, 48, 32), 2, 2),
    ((64, 32, 16), 4, 4), ((37, 21, 14), 1, 1), ((37, 21, 14), 2, 1), ((30, 22, 18), 4, 1), ((6, 6, 6), 2, 2),
]


@pytest.mark.parametrize("dims,eb,nc", MIP_CASES)
def test_mip_level_matches_oracle(gc, orc, torch_cuda, dims, eb, nc):
    torch = torch_cuda
    rng = np.random.default_rng(dims[0] * 7 + eb)
    n = dims[0] * dims[1] * dims[2] * eb
    cb = eb // nc
    if cb == 4:
        src = rng.standard_normal(n // 4).astype(np.float32) * 1000
        raw = src.view(np.uint8)
    else:
        raw = rng.integers(0, 256, n, dtype=np.uint8)
        src = raw.view({1: np.uint8, 2: np.uint16}[cb])
    d_src = torch.from_numpy(raw.copy()).cuda()
    out_n = (dims[0] // 2) * (dims[1] // 2) * (dims[2] // 2) * eb
    d_dst = torch.zeros(out_n, dtype=torch.uint8, device="cuda")
    gc.Mipmapper.down_scale(d_src.data_ptr(), d_dst.data_ptr(), dims, eb, nc)
    ref = orc.mip_level(src, dims, eb, nc).view(np.uint8)
    assert np.array_equal(to_np(d_dst), ref)


def test_mip_full_size_floor_mean_property(gc, torch_cuda):
    """1024^3 u8 (1 GiB): every output voxel is floor(sum of its 8 inputs / 8),
    checked with an independent torch reduction, slab by slab."""
    torch = torch_cuda
    X = Y = Z = 1024
    src = torch.randint(0, 256, (Z, Y, X), dtype=torch.uint8, device="cuda")
    dst = torch.empty((Z // 2, Y // 2, X // 2), dtype=torch.uint8, device="cuda")
    gc.Mipmapper.down_scale(src.data_ptr(), dst.data_ptr(), (X, Y, Z), 1, 1)
    torch.cuda.synchronize()
    for z0 in range(0, Z, 128):
        s = src[z0:z0 + 128].to(torch.int32).reshape(64, 2, Y // 2, 2, X // 2, 2).sum(dim=(1, 3, 5))
        assert torch.equal((s // 8).to(torch.uint8), dst[z0 // 2:z0 // 2 + 64])


BRICK_CASES = [
    # size, bpc, channels, B, c, big brick
    ((64, 64, 64), 1, 1, 16, 1, (1, 1, 1)),
    ((64, 56, 48), 2, 1, 16, 1, (1, 1, 1)),
    ((70, 50, 40), 2, 1, 32, 1, (1, 1, 1)),
    ((48, 40, 36), 1, 2, 16, 2, (2, 2, 2)),
    ((50, 30, 45), 1, 1, 8, 1, (2, 1, 3)),
    # 16-byte row path of the bricker at every start offset: covering 2 with
    # B32 u16, covering 0, and 4-byte voxels (two u16 channels) in big bricks
    ((96, 80, 64), 2, 1, 32, 2, (1, 1, 1)),
    ((64, 64, 32), 1, 1, 16, 0, (1, 1, 1)),
    ((64, 48, 40), 2, 2, 16, 1, (1, 2, 1)),
]


@pytest.mark.parametrize("size,bpc,ch,B,c,bb", BRICK_CASES)
def test_pre_process_matches_oracle(gc, orc, torch_cuda, size, bpc, ch, B, c, bb):
    """Mip pyramid + bricks of every level (Application::pre_process) on the
    device equal the oracle's restatement of Mipmapper + process_bricking."""
    vol = gc.volume_desc(size, B, c, bpc * ch, ch, bb)
    layout = gc.compute_layout(vol)
    if any(tuple(layout.mip[l]) != tuple(layout.initial[l]) for l in range(layout.nb_levels)):
        pytest.skip("geometry with levels that stop halving")
    d = scenario.gpu_volume(gc, torch_cuda, size, bpc, 21, 5, channels=ch)
    store, offs, _ = gc.pre_process(vol, layout, d)
    o = scenario.orc_volume(orc, size, bpc, 21, 5, channels=ch)
    ref, roffs = scenario.orc_store(orc, gc, o.reshape(-1).view(np.uint8), vol, layout)
    assert list(offs) == list(roffs)
    assert np.array_equal(store.numpy(), ref)


def test_empty_flags_match_oracle(gc, orc, torch_cuda):
    size, B = (64, 64, 64), 16
    vol = gc.volume_desc(size, B, 1, 1, 1)
    layout = gc.compute_layout(vol)
    d = scenario.gpu_volume(gc, torch_cuda, size, 1, 3, 3)
    store, offs, keys = gc.pre_process(vol, layout, d, empty_threshold=45.0)
    big = B ** 3
    want = []
    for l in range(layout.nb_levels):
        nb = layout.nb_big_bricks[l]
        n = nb[0] * nb[1] * nb[2]
        flags = orc.empty_flags(store.numpy()[offs[l]:offs[l] + n * big], n, big, 1, 45.0)
        for i in np.nonzero(flags)[0]:
            want.append(gc.brick_key(l, int(i % nb[0]), int((i // nb[0]) % nb[1]), int(i // (nb[0] * nb[1]))))
    assert sorted(keys) == sorted(want) and len(want) > 0
