"""The device-side handle of the cache (gc_cache_device_view +
gc_sample_normalized of include/gc_cache_device.cuh), used from a user's own
kernel (tests/user_sampler.cu, compiled here with nvcc) the way the
reference's K_CacheManager<T>::get_normalized is used
(K_CacheManager.hpp:61-71, 265-361): statuses, sampled values, usage stamps
and brick requests equal the oracle's fetch of the same samples, bit for bit."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import scenario

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def user_lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("user") / "libuser_sampler.so")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-shared", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "user_sampler.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    lib.user_sample.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int] + [ctypes.c_void_p] * 2
    return lib


@pytest.mark.parametrize("bpc", [1, 2])
def test_user_kernel_samples_like_the_oracle(gc, orc, torch_cuda, user_lib, bpc):
    torch = torch_cuda
    size = (64, 64, 64)
    vol = gc.volume_desc(size, 16, 1, bpc, 1)
    layout = gc.compute_layout(vol)
    d = scenario.gpu_volume(gc, torch, size, bpc, 5, 6)
    store, offs, _ = gc.pre_process(vol, layout, d)
    cm = gc.CacheManager(vol, layout, (6, 6, 6), max_requests=40, sync_loader=True)
    cm.set_source_host(store, offs)
    # a few frames of a view: part of the bricks resident, the rest not
    W = H = 48
    tf = scenario.ramp_tf()
    tf_dev = torch.from_numpy(tf.reshape(-1).copy()).cuda()
    bufs = [torch.zeros(W * H, dtype=torch.int32, device="cuda"), torch.zeros(W * H, dtype=torch.float32, device="cuda"),
            torch.zeros(W * H * 4, dtype=torch.float32, device="cuda")]
    view = gc.make_view(scenario.orbit_camera(gc, 1, 8, 2.5), W, H, tf_dev.data_ptr(), 256, *[b.data_ptr() for b in bufs])
    for _ in range(4):
        cm.render(view)
        cm.update()
    # the oracle holds the same cache state
    oc = orc.Cache(cm.desc)
    cm.dump(gc.DUMP_MRPD, oc.mrpd())
    cm.dump(gc.DUMP_POOL, oc.pool())
    cm.dump(gc.DUMP_USAGE, oc.usage())
    cm.dump(gc.DUMP_REQUESTS, oc.requests())
    oc.timestamp = cm.timestamp()
    v = cm.device_view()
    assert v.timestamp == cm.timestamp() and v.n_levels == layout.nb_levels
    rng = np.random.default_rng(bpc)
    n = 20000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.0, 0.99, (n, 3))
    pos[:, 3] = rng.integers(0, layout.nb_levels, n)
    d_pos = torch.from_numpy(pos).cuda()
    d_val = torch.zeros(n, dtype=torch.float32, device="cuda")
    d_st = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    assert user_lib.user_sample(ctypes.addressof(v), d_pos.data_ptr(), n, d_val.data_ptr(), d_st.data_ptr()) == 0
    want = [oc.sample_normalized(int(p[3]), float(p[0]), float(p[1]), float(p[2])) for p in pos]
    st = d_st.cpu().numpy()
    val = d_val.cpu().numpy()
    want_st = np.array([w[0] for w in want])
    want_val = np.array([w[1] for w in want], np.float32)
    assert np.array_equal(st, want_st)
    mapped = st == 0
    assert mapped.any() and (st == 1).any(), "samples of resident and of missing bricks"
    assert np.array_equal(val[mapped], want_val[mapped])  # bit-exact values
    # side effects: the usage stamps and brick requests of those samples
    for what, ref in ((gc.DUMP_USAGE, oc.usage()), (gc.DUMP_REQUESTS, oc.requests())):
        got = cm.dump(what, np.zeros_like(ref))
        assert np.array_equal(got, ref), what
    cm.close()
    oc.close()
