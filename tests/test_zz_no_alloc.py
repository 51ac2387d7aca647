"""sphx_density_noalloc: the density evaluation for callers that cannot allocate device
memory (an application that owns the whole device-memory budget, or a frame loop that
cannot take the synchronisation of cudaMalloc/cudaFree).  Its working memory is one
fixed device array inside the library, shared by every call.

Checked through the C ABI against the context entry points (sphx_eval + sphx_download)
on two calls in a row with different inputs -- the second call must not see anything of
the first one's -- within the tolerance of the other GPU tests: bit-identical.  The
caller-side buffers here come from torch; the entry point itself allocates nothing.
This file is collected last so that a run stopping at the first failure has already run
every other test.
"""
import numpy as np
import pytest

import sph_oracle as O
import sphx
import sphx_inputs as I

pytestmark = pytest.mark.gpu


def context_density(w):
    ctx = sphx.Context(w.n)
    ctx.set_params(w.params)
    ctx.upload(w.pos, w.vel, w.mass)
    ctx.eval()
    out = ctx.download(pos=False, vel=False, acc=False)
    ctx.close()
    return out["rho"], out["pressure"]


def noalloc_density(torch, w):
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(np.ascontiguousarray(w.pos)).to(dev)
    mass = torch.from_numpy(np.ascontiguousarray(w.mass)).to(dev)
    rho = torch.full((w.n,), float("nan"), dtype=torch.float32, device=dev)
    prs = torch.full((w.n,), float("nan"), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sphx.density_noalloc(w.params, w.n, pos.data_ptr(), mass.data_ptr(), rho.data_ptr(),
                         prs.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize(dev)
    return rho.cpu().numpy(), prs.cpu().numpy()


def cluster_workload():
    rng = np.random.default_rng(21)
    pos = np.concatenate([
        (0.3 + rng.random((30000, 3)) * 0.25).astype(np.float32),
        np.array([[50.0, -20.0, 7.0]], np.float32) + (rng.random((2000, 3)) * 0.1).astype(np.float32),
    ])
    n = pos.shape[0]
    prm = I.params16(xmin=-100, xmax=100, ymin=-100, ymax=100, zmin=-100, zmax=100)
    return I.Workload(name="clusters_32k", pos=pos, vel=np.zeros((n, 3), np.float32),
                      mass=np.full(n, 1.2e-3, np.float32), params=prm, dt=1e-3, steps=1)


def test_noalloc_density_matches_context_path_on_two_calls():
    torch = pytest.importorskip("torch")
    first = I.config0()               # 10,000-particle dam break
    second = cluster_workload()       # 32,000 particles over a far larger, folded box
    for w in (first, second):
        rho_ref, p_ref = context_density(w)
        rho, prs = noalloc_density(torch, w)
        assert O.bits_equal(rho, rho_ref), O.mismatch_report(rho, rho_ref, f"rho {w.name}")
        assert O.bits_equal(prs, p_ref), O.mismatch_report(prs, p_ref, f"P {w.name}")


def test_noalloc_rejects_sizes_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    n = sphx.NOALLOC_MAX_PARTICLES + 1
    dev = torch.device("cuda", 0)
    pos = torch.zeros((n, 3), dtype=torch.float32, device=dev)
    mass = torch.ones((n,), dtype=torch.float32, device=dev)
    rho = torch.zeros((n,), dtype=torch.float32, device=dev)
    with pytest.raises(sphx.SphxError) as ei:
        sphx.density_noalloc(I.params16(), n, pos.data_ptr(), mass.data_ptr(), rho.data_ptr(), None)
    assert ei.value.code == -5


def test_noalloc_second_call_takes_no_device_memory():
    """After a first call on the device (which looks up the array's address and loads
    the kernels), further calls leave the device's free memory exactly as it was: the
    working memory is the library's fixed array, nothing is allocated per call."""
    torch = pytest.importorskip("torch")
    w = cluster_workload()
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(np.ascontiguousarray(w.pos)).to(dev)
    mass = torch.from_numpy(np.ascontiguousarray(w.mass)).to(dev)
    rho = torch.empty((w.n,), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def call():
        sphx.density_noalloc(w.params, w.n, pos.data_ptr(), mass.data_ptr(), rho.data_ptr(),
                             None, stream.cuda_stream)
        torch.cuda.synchronize(dev)

    call()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(3):
        call()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, (free0, free1)
