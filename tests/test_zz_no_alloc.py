"""mc_transport_bank_noalloc: the bank transport for callers that cannot
allocate device memory (while recording a CUDA graph, or under a device
memory budget fixed at start-up).  Through the C ABI, two calls in a row
must bank exactly the sites the allocating entry point (mc_transport_bank)
banks, with the same tallies; oversized calls are refused.

Collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test.
"""
import numpy as np
import pytest

from minimc_gb300 import RNG_MINSTD, RNG_PHILOX, SITE_DTYPE, Context, MCError, synth

pytestmark = pytest.mark.gpu
FP_RTOL = 1e-12  # tallies: summation order only


def start_sites(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    s = np.zeros(n, SITE_DTYPE)
    s["x"], s["y"], s["z"] = (rng.uniform(-5, 5, n) for _ in range(3))
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    st = np.sqrt(1 - mu * mu)
    s["u"], s["v"], s["w"] = mu, st * np.cos(ph), st * np.sin(ph)
    s["energy"] = 1.0
    s["key"] = np.arange(1, n + 1, dtype=np.uint64)
    return s


@pytest.mark.parametrize("rng", [RNG_PHILOX, RNG_MINSTD])
def test_noalloc_matches_allocating_entry_point(rng, built_library):
    import torch

    xml = synth.one_group_cube(histories=1000).xml()
    ref = Context(0)
    ref.load_xml(xml)
    noa = Context(0)
    noa.load_xml(xml)
    n = 12000
    cap = n * noa.info.max_yield
    d_in = torch.empty(n * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_out = torch.empty(cap * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    sites = start_sites(n, 11)
    for call in range(2):
        expect = ref.transport_bank(sites, rng=rng, fast_math=1)
        d_in.copy_(torch.from_numpy(sites.view(np.uint8)).to("cuda"))
        torch.cuda.synchronize()
        m = noa.transport_bank_noalloc(d_in.data_ptr(), n, d_out.data_ptr(), cap, rng=rng, fast_math=1)
        got = d_out[: m * SITE_DTYPE.itemsize].cpu().numpy().view(SITE_DTYPE)
        assert m == len(expect) > 0, call
        assert np.array_equal(got.view(np.uint8), expect.view(np.uint8)), call
        s_ref, q_ref = ref.tallies()
        s_noa, q_noa = noa.tallies()
        np.testing.assert_allclose(s_noa, s_ref, rtol=FP_RTOL)
        np.testing.assert_allclose(q_noa, q_ref, rtol=FP_RTOL)
        # next call: resampled bank, new stream keys
        pick = np.random.default_rng(call).integers(0, m, n)
        sites = expect[pick].copy()
        sites["key"] = np.arange(n, dtype=np.uint64) + (call + 2) * n


def test_noalloc_refuses_oversized_calls(built_library):
    import torch

    ctx = Context(0)
    ctx.load_xml(synth.one_group_cube(histories=1000).xml())
    d = torch.empty(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(MCError) as e:
        ctx.transport_bank_noalloc(d.data_ptr(), 16385, d.data_ptr(), 1)
    assert e.value.code == -1 and "exceed the limit of 16384" in e.value.message


def _raw_call(ctx, d_in: int, n: int, d_out: int, cap: int, **kw) -> tuple[int, int]:
    """The C call itself: its status and the bank size it reports, which the
    Context wrapper would turn into an exception on an overflow."""
    import ctypes as C

    o = ctx.opts(**kw)
    n_out = C.c_uint64()
    rc = ctx.lib.mc_transport_bank_noalloc(ctx.h, C.c_void_p(d_in), n, C.byref(o), C.c_void_p(d_out), cap,
                                           C.byref(n_out))
    return rc, int(n_out.value)


def test_noalloc_overflow_keeps_the_first_cap_sites(built_library):
    import torch

    xml = synth.one_group_cube(histories=1000).xml()
    ref = Context(0)
    ref.load_xml(xml)
    noa = Context(0)
    noa.load_xml(xml)
    n = 4000
    sites = start_sites(n, 23)
    expect = ref.transport_bank(sites, rng=RNG_PHILOX, fast_math=1)
    m = len(expect)
    cap = m // 2
    d_in = torch.from_numpy(sites.view(np.uint8).copy()).to("cuda")
    guard = 64  # sites past cap that must stay untouched
    d_out = torch.full(((cap + guard) * SITE_DTYPE.itemsize,), 0xA5, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc, got_m = _raw_call(noa, d_in.data_ptr(), n, d_out.data_ptr(), cap, rng=RNG_PHILOX, fast_math=1)
    assert rc == -8 and got_m == m  # MC_ERR_OVERFLOW with the full bank size
    out = d_out.cpu().numpy()
    got = out[: cap * SITE_DTYPE.itemsize].view(SITE_DTYPE)
    assert np.array_equal(got.view(np.uint8), expect[:cap].view(np.uint8))
    assert np.all(out[cap * SITE_DTYPE.itemsize:] == 0xA5)
    # the context stays usable
    d_big = torch.empty(n * noa.info.max_yield * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    assert noa.transport_bank_noalloc(d_in.data_ptr(), n, d_big.data_ptr(), n * noa.info.max_yield,
                                      rng=RNG_PHILOX, fast_math=1) > 0


def test_noalloc_refuses_large_yields_and_continuous_energy(tmp_path, built_library):
    import torch

    from minimc_gb300 import synth_ce

    d = torch.empty(1024 * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    big = Context(0)
    big.load_xml(synth.infinite_medium(c=0.2, capture=0.6, fission=0.2, nubar=4.5, histories=100, keig=(1, 1)).xml())
    assert big.info.max_yield > 4
    with pytest.raises(MCError) as e:
        big.transport_bank_noalloc(d.data_ptr(), 10, d.data_ptr(), 100)
    assert e.value.code == -1 and "mean secondaries per fission" in e.value.message
    nuc = synth_ce.write_flat_nuclide(tmp_path, "A", 1.0, 0.1, 1.0, fission=0.3, nubar=2.4,
                                      energies=np.geomspace(1e-11, 20, 7))
    ce = Context(0)
    ce.load_xml(synth_ce.ce_problem_xml({"A": nuc}, histories=10, names=("A",), afrac=(1.0,)), str(tmp_path))
    with pytest.raises(MCError) as e:
        ce.transport_bank_noalloc(d.data_ptr(), 10, d.data_ptr(), 100)
    assert e.value.code == -1 and "multigroup problems only" in e.value.message


def test_noalloc_refuses_pageable_host_buffers(built_library):
    import torch

    ctx = Context(0)
    ctx.load_xml(synth.one_group_cube(histories=1000).xml())
    host = start_sites(16, 3)  # pageable numpy memory: not reachable by the kernels
    d = torch.empty(64 * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    with pytest.raises(MCError) as e:
        ctx.transport_bank_noalloc(host.ctypes.data, 16, d.data_ptr(), 64)
    assert e.value.code == -1 and "not device or page-locked memory" in e.value.message
    with pytest.raises(MCError) as e:
        ctx.transport_bank_noalloc(d.data_ptr(), 16, host.ctypes.data, 16)
    assert e.value.code == -1 and "fission_sites is not device" in e.value.message
