"""GPU transport parity, through the C ABI.

* Reference streams (minstd): a GPU history draws the same random numbers as
  the reference would, so fission banks (k per cycle), per-history event
  counts and integer tallies equal the CPU oracle's exactly; floating-point
  tallies agree to the last few ulps (summation order).
* Philox streams: statistical agreement (k within 3 combined sigma) and
  run-to-run / schedule-to-schedule reproducibility.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from minimc_gb300 import (BANK_DIRECT, BANK_SLOTS, GEOMETRY_REFERENCE, RNG_MINSTD, RNG_PHILOX, SCHEDULE_EVENT,
                          SCHEDULE_HISTORY, Context, MCError, synth)
from oracle.build import Oracle

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
KA = json.loads((GOLDEN / "reference_known_answers.json").read_text())
FP_RTOL = 1e-12  # floating-point tallies: summation order only


def gpu_ctx(xml, mode=None):
    ctx = Context(0)
    if mode is not None:
        ctx.set_geometry_mode(mode)
    ctx.load_xml(xml)
    return ctx


@pytest.mark.parametrize("schedule", [SCHEDULE_HISTORY, SCHEDULE_EVENT])
def test_keig_one_group_cube_identical_to_oracle(schedule, built_library):
    p = synth.one_group_cube(histories=20000, inactive=5, active=10)
    xml = p.xml()
    g = gpu_ctx(xml).run_keigenvalue(rng=RNG_MINSTD, schedule=schedule)
    o = Oracle(xml).run_keigenvalue(20000, 1, 5, 10, threads=8)
    assert np.array_equal(g.bank_size, o["bank_size"])
    assert np.array_equal(g.k_cycle, o["k_cycle"])
    np.testing.assert_allclose(g.sum, o["sum"], rtol=FP_RTOL)
    np.testing.assert_allclose(g.sum_sq, o["sum_sq"], rtol=FP_RTOL)


def test_keig_two_zone_identical_to_oracle(built_library):
    p = synth.two_zone_cubes(histories=50000, inactive=3, active=3)
    xml = p.xml()
    g = gpu_ctx(xml).run_keigenvalue(rng=RNG_MINSTD)
    o = Oracle(xml).run_keigenvalue(50000, 1, 3, 3, threads=8)
    assert np.array_equal(g.bank_size, o["bank_size"])
    np.testing.assert_allclose(g.sum, o["sum"], rtol=FP_RTOL)


@pytest.mark.parametrize("schedule", [SCHEDULE_HISTORY, SCHEDULE_EVENT])
def test_fixed_source_with_secondaries_per_history(schedule, built_library):
    """Fixed source in a fissile sphere: secondaries are transported inside
    their history; per-history events and fates equal the oracle's."""
    p = synth.one_group_cube(histories=20000)
    p.problem = "fixedsource"
    p.nuclides[0].nubar = np.array([0.9])  # subcritical
    xml = p.xml()
    n = 20000
    g = gpu_ctx(xml).run_fixed_source(rng=RNG_MINSTD, per_history=True, histories=n, schedule=schedule)
    o = Oracle(xml).run_fixed_source(n, 1, threads=8, per_history=True)
    assert g.raw.secondaries == o["secondaries"] > 0
    assert np.array_equal(g.history_events, o["history_events"])
    assert np.array_equal(g.history_fate, o["history_fate"])
    np.testing.assert_allclose(g.sum, o["sum"], rtol=FP_RTOL)


def test_point_source_leakage_reference_test(built_library):
    """The reference's statistical test (leakage = e^-1 within 3 sigma) on
    both random streams; with minstd the count equals the oracle's."""
    ka = KA["point_source_leakage"]
    xml = (GOLDEN / "point_source_leakage.xml").read_text()
    p, n = ka["expected"], ka["histories"]
    o = Oracle(xml).run_fixed_source(n, 1)
    for rng in (RNG_MINSTD, RNG_PHILOX):
        r = gpu_ctx(xml).run_fixed_source(rng=rng)
        est = r.sum[0] / n
        assert abs(est - p) / p < 3 * math.sqrt((1 - p) / (p * n))
        if rng == RNG_MINSTD:
            assert r.sum[0] == o["sum"][0]


def test_result_file(built_library, tmp_path):
    """Driver.write_output: the .out file beside the input holds the result
    text for the GPU's tallies; with reference streams those tallies equal
    the oracle's, so the file equals the text of the oracle's sums (which
    the CPU suite pins on the reference's own output)."""
    from minimc_gb300.engine import Driver, format_output

    xml = (GOLDEN / "point_source_leakage.xml").read_text()
    path = tmp_path / "leakage.xml"
    path.write_text(xml)
    n = KA["point_source_leakage"]["histories"]
    drv = Driver.create(path)
    r = drv.solve(rng=RNG_MINSTD)
    out = drv.write_output(r, path)
    assert out == tmp_path / "leakage.out"
    o = Oracle(xml).run_fixed_source(n, 1)
    assert out.read_text() == format_output(xml, GOLDEN, o["sum"], o["sum_sq"], n)
    assert out.read_text().startswith(f"{n}\n\nleakage\n")


def test_reference_geometry_mode_fixed_source(built_library):
    xml = (GOLDEN / "mg_spheres.xml").read_text()
    n = 50000
    g = gpu_ctx(xml, GEOMETRY_REFERENCE).run_fixed_source(rng=RNG_MINSTD, per_history=True, histories=n)
    oc = Oracle(xml)
    oc.set_quirks(True)
    o = oc.run_fixed_source(n, 1, threads=8, per_history=True)
    agree = np.mean((g.history_events == o["history_events"]) & (g.history_fate == o["history_fate"]))
    assert agree > 0.999  # libm ulps may move a grazing history
    assert abs(g.sum[0] - o["sum"][0]) <= 0.001 * n


def test_philox_keig_matches_oracle_statistically(built_library):
    p = synth.one_group_cube(histories=20000, inactive=10, active=30)
    xml = p.xml()
    for fast in (0, 1):
        g = gpu_ctx(xml).run_keigenvalue(rng=RNG_PHILOX, fast_math=fast)
        o = Oracle(xml).run_keigenvalue(20000, 1, 10, 30, threads=8)
        kg, ko = g.k_cycle[10:], o["k_cycle"][10:]
        sig = math.sqrt(kg.var(ddof=1) / len(kg) + ko.var(ddof=1) / len(ko))
        assert abs(kg.mean() - ko.mean()) < 3 * sig + 1e-4, (fast, kg.mean(), ko.mean(), sig)


def test_reflected_box_gives_k_inf(built_library):
    p = synth.one_group_cube(histories=100000, inactive=5, active=20)
    p.surfaces = synth.box_planes("cube", 10.0, reflective=True)
    r = gpu_ctx(p.xml()).run_keigenvalue(rng=RNG_PHILOX, fast_math=1)
    k = r.k_cycle[5:]
    assert r.raw.lost == 0
    assert k.mean() == pytest.approx(5 / 3, abs=4 * k.std(ddof=1) / math.sqrt(len(k)) + 2e-4)


def test_philox_reproducible_and_schedule_independent(built_library):
    p = synth.two_zone_cubes(histories=200000, inactive=2, active=2)
    xml = p.xml()
    runs = [gpu_ctx(xml).run_keigenvalue(rng=RNG_PHILOX, fast_math=1, schedule=s)
            for s in (SCHEDULE_HISTORY, SCHEDULE_HISTORY, SCHEDULE_EVENT)]
    for r in runs[1:]:
        assert np.array_equal(r.bank_size, runs[0].bank_size)
        np.testing.assert_allclose(r.sum, runs[0].sum, rtol=FP_RTOL)


def test_event_schedule_sorted_queues_identical(built_library):
    """Collision queues counting-sorted by (type, material, group) before
    every collide step give the same banks and tallies as the unsorted
    event schedule and the history schedule: each particle draws from its
    own stream, so the processing order changes nothing."""
    p = synth.two_zone_cubes(histories=200000, inactive=2, active=2)
    xml = p.xml()
    hist = gpu_ctx(xml).run_keigenvalue(rng=RNG_PHILOX, fast_math=1, schedule=SCHEDULE_HISTORY)
    for sort_min in (0xFFFFFFFF, 1, 50000):
        ev = gpu_ctx(xml).run_keigenvalue(rng=RNG_PHILOX, fast_math=1, schedule=SCHEDULE_EVENT,
                                          queue_sort_min=sort_min)
        assert np.array_equal(ev.bank_size, hist.bank_size), sort_min
        np.testing.assert_allclose(ev.sum, hist.sum, rtol=FP_RTOL)
    # fixed source with secondaries in their history
    fs = synth.one_group_cube(histories=20000, side=2.0)  # small: about one secondary per history
    fs.problem = "fixedsource"
    xf = fs.xml()
    a = gpu_ctx(xf).run_fixed_source(rng=RNG_PHILOX, fast_math=1, schedule=SCHEDULE_EVENT, queue_sort_min=1)
    b = gpu_ctx(xf).run_fixed_source(rng=RNG_PHILOX, fast_math=1, schedule=SCHEDULE_HISTORY)
    assert a.raw.events == b.raw.events and a.raw.secondaries == b.raw.secondaries
    np.testing.assert_allclose(a.sum, b.sum, rtol=FP_RTOL)


def test_autotuner_candidates(built_library):
    """MC_SCHEDULE_AUTO on a k-eigenvalue run: the tuner times the history
    kernel's five occupancy variants at blocks of 256 and 128 and the event
    schedule with unsorted and sorted collision queues, then keeps the
    default (variant 1 at 256 threads) unless a candidate beats it by more
    than 3 %; the run's results do not depend on the choice."""
    p = synth.two_zone_cubes(histories=200000, inactive=3, active=2)
    ctx = gpu_ctx(p.xml())
    r = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=1)
    info = ctx.schedule_info()
    t = info["tune_kernel_ms"]
    assert len(t) == 12, info
    assert info["schedule"] in ("history", "event") and info["block"] in (128, 256)
    default = info["schedule"] == "history" and info["variant"] == 1 and info["block"] == 256
    assert default or min(t) < 0.97 * t[1], info
    ref = gpu_ctx(p.xml()).run_keigenvalue(rng=RNG_PHILOX, fast_math=1, schedule=SCHEDULE_HISTORY, variant=1)
    assert np.array_equal(r.bank_size, ref.bank_size)
    np.testing.assert_allclose(r.sum, ref.sum, rtol=FP_RTOL)


def test_full_size_two_zone_invariants(built_library):
    """1e6 histories per cycle: no lost particles, fission bank = sum of
    per-history sites, tallies finite and non-negative, k in range."""
    p = synth.two_zone_cubes(histories=1_000_000, inactive=2, active=2)
    r = gpu_ctx(p.xml()).run_keigenvalue(rng=RNG_PHILOX, fast_math=1)
    assert r.raw.lost == 0 and r.raw.overflow == 0 and r.raw.capped == 0
    assert np.all(np.isfinite(r.sum)) and np.all(r.sum >= 0) and np.all(r.sum_sq >= 0)
    assert np.all((r.k_cycle > 0.7) & (r.k_cycle < 1.3))
    assert r.raw.events > 5 * 4 * 1_000_000


def test_event_cap_reports_and_context_survives(built_library):
    """Per-particle event cap: the run stops those particles, reports
    MC_ERR_EVENT_CAP, and the context keeps working."""
    xml = (GOLDEN / "infinite_medium.xml").read_text()
    ctx = gpu_ctx(xml)
    with pytest.raises(MCError) as e:
        ctx.run_fixed_source(rng=RNG_PHILOX, histories=10000, max_events=1)
    assert e.value.code == -9
    r = ctx.run_fixed_source(rng=RNG_PHILOX, histories=10000)
    assert r.raw.capped == 0 and r.raw.lost == 0


def test_lost_particle_reported(built_library):
    """A source outside every cell: the reference throws; the engine reports
    MC_ERR_LOST with the reference's message."""
    xml = (GOLDEN / "mg_spheres.xml").read_text().replace(
        '<void><surface name="outer shell" sense="+1"/></void>', "").replace(
        '<constant x="0" y="0" z="0"/>', '<constant x="5" y="0" z="0"/>')
    ctx = gpu_ctx(xml)
    with pytest.raises(MCError) as e:
        ctx.run_fixed_source(rng=RNG_PHILOX, histories=100)
    assert e.value.code == -5 and "Point does not belong to any Cell" in e.value.message


def test_transport_bank_pinned_sites_read_in_place(built_library):
    """mc_transport_bank reads sites in page-locked host memory in place
    (copies pageable ones first): with page-locked or pageable inputs and
    outputs it gives the same fission bank, and a too-small output is not
    overrun."""
    import ctypes as C

    import torch

    from minimc_gb300 import SITE_DTYPE

    p = synth.two_zone_cubes(histories=20000, groups=4)
    ctx = gpu_ctx(p.xml())
    n = 20000
    rng = np.random.default_rng(3)
    sites = np.zeros(n, SITE_DTYPE)
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    sites["u"], sites["v"], sites["w"] = mu, np.sqrt(1 - mu * mu) * np.cos(ph), np.sqrt(1 - mu * mu) * np.sin(ph)
    sites["x"] = rng.uniform(-10, 10, n)
    sites["energy"] = 1.0
    sites["key"] = np.arange(n, dtype=np.uint64) + 1
    pinned = torch.empty(n * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(SITE_DTYPE)
    pinned[:] = sites
    cap = n * max(1, ctx.info.max_yield)

    def pinned_out(k):
        return torch.empty(k * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(SITE_DTYPE)

    out1 = np.zeros(cap, SITE_DTYPE)
    m1 = ctx.transport_bank_into(sites, out1, rng=RNG_MINSTD)
    assert m1 > 0
    for src, out in ((pinned, np.zeros(cap, SITE_DTYPE)), (sites, pinned_out(cap)), (pinned, pinned_out(cap))):
        m = ctx.transport_bank_into(src, out, rng=RNG_MINSTD)
        assert m == m1
        assert np.array_equal(out[:m], out1[:m1])
    # a page-locked output of half the bank: the call reports the overflow,
    # writes the first half and nothing past it
    half = m1 // 2
    guard = pinned_out(half + 64)
    guard[:] = np.zeros(1, SITE_DTYPE)
    guard["key"][half:] = 0xABCDEF
    with pytest.raises(MCError):
        ctx.check(ctx.lib.mc_transport_bank(ctx.h, pinned.ctypes.data_as(C.c_void_p), n,
                                            C.byref(ctx.opts(rng=RNG_MINSTD)), guard.ctypes.data_as(C.c_void_p),
                                            half, C.byref(C.c_uint64())))
    assert np.array_equal(guard[:half], out1[:half])
    assert (guard["key"][half:] == 0xABCDEF).all()


def _bank_sites(n, seed):
    rng = np.random.default_rng(seed)
    from minimc_gb300 import SITE_DTYPE

    sites = np.zeros(n, SITE_DTYPE)
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    sites["u"], sites["v"], sites["w"] = mu, np.sqrt(1 - mu * mu) * np.cos(ph), np.sqrt(1 - mu * mu) * np.sin(ph)
    sites["x"] = rng.uniform(-10, 10, n)
    sites["energy"] = 1.0
    sites["key"] = np.arange(n, dtype=np.uint64) + 7
    return sites


@pytest.mark.parametrize("fast", [0, 1])
def test_bank_direct_path_equals_slot_path(fast, built_library):
    """Philox fission sites sampled straight into their bank positions (into
    page-locked host memory in place, or into the device bank) equal the
    per-history slots + compaction path site for site; a too-small
    page-locked output is filled to its end and not overrun."""
    import ctypes as C

    import torch

    from minimc_gb300 import SITE_DTYPE

    p = synth.two_zone_cubes(histories=20000, groups=4)
    ctx = gpu_ctx(p.xml())
    n = 20000
    sites = _bank_sites(n, 5)
    cap = n * max(1, ctx.info.max_yield)

    def pinned(k):
        return torch.empty(k * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(SITE_DTYPE)

    opts = dict(rng=RNG_PHILOX, fast_math=fast)
    ref = np.zeros(cap, SITE_DTYPE)
    m0 = ctx.transport_bank_into(sites, ref, bank_path=BANK_SLOTS, **opts)
    assert m0 > 0
    for path, out in ((BANK_SLOTS, pinned(cap)), (BANK_DIRECT, np.zeros(cap, SITE_DTYPE)), (BANK_DIRECT, pinned(cap))):
        m = ctx.transport_bank_into(sites, out, bank_path=path, **opts)
        assert m == m0
        assert np.array_equal(out[:m].view(np.uint8), ref[:m0].view(np.uint8))
    half = m0 // 2
    guard = pinned(half + 64)
    guard[:] = np.zeros(1, SITE_DTYPE)
    guard["key"][half:] = 0xABCDEF
    with pytest.raises(MCError):
        ctx.check(ctx.lib.mc_transport_bank(ctx.h, sites.ctypes.data_as(C.c_void_p), n,
                                            C.byref(ctx.opts(bank_path=BANK_DIRECT, **opts)),
                                            guard.ctypes.data_as(C.c_void_p), half, C.byref(C.c_uint64())))
    assert np.array_equal(guard[:half].view(np.uint8), ref[:half].view(np.uint8))
    assert (guard["key"][half:] == 0xABCDEF).all()


@pytest.mark.parametrize("fast", [0, 1])
def test_bank_direct_path_many_sites_per_cta(fast, built_library):
    """A high-yield problem (one group, nu = 7.5, fission 70 % of
    collisions): a CTA's 128 histories yield several hundred sites, so the
    per-site kernel stages them through many 128-site windows; the direct
    bank equals the slot path's byte for byte, in device and page-locked
    memory, and a capacity ending inside a window keeps exactly the first
    sites."""
    import ctypes as C

    import torch

    from minimc_gb300 import SITE_DTYPE
    from minimc_gb300.synth import MGNuclide

    p = synth.one_group_cube(histories=20000, inactive=1, active=1)
    p.nuclides = [MGNuclide("fuel", capture=np.array([0.1]), scatter=np.array([[0.2]]), fission=np.array([0.7]),
                            nubar=np.array([7.5]), chi=np.array([[1.0]]))]
    ctx = gpu_ctx(p.xml())
    assert ctx.info.max_yield == 8
    n = 20000
    sites = _bank_sites(n, 11)
    cap = n * ctx.info.max_yield

    def pinned(k):
        return torch.empty(k * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(SITE_DTYPE)

    opts = dict(rng=RNG_PHILOX, fast_math=fast)
    ref = np.zeros(cap, SITE_DTYPE)
    m0 = ctx.transport_bank_into(sites, ref, bank_path=BANK_SLOTS, **opts)
    assert m0 > 3 * n  # several sites per history: many windows per CTA
    for out in (np.zeros(cap, SITE_DTYPE), pinned(cap)):
        m = ctx.transport_bank_into(sites, out, bank_path=BANK_DIRECT, **opts)
        assert m == m0
        assert np.array_equal(out[:m].view(np.uint8), ref[:m0].view(np.uint8))
    part = m0 // 3 + 37  # inside some CTA's window
    guard = pinned(part + 64)
    guard[:] = np.zeros(1, SITE_DTYPE)
    guard["key"][part:] = 0xABCDEF
    with pytest.raises(MCError):
        ctx.check(ctx.lib.mc_transport_bank(ctx.h, sites.ctypes.data_as(C.c_void_p), n,
                                            C.byref(ctx.opts(bank_path=BANK_DIRECT, **opts)),
                                            guard.ctypes.data_as(C.c_void_p), part, C.byref(C.c_uint64())))
    assert np.array_equal(guard[:part].view(np.uint8), ref[:part].view(np.uint8))
    assert (guard["key"][part:] == 0xABCDEF).all()


def test_bank_direct_path_keig_cycles(built_library):
    """k-eigenvalue cycles give the same bank sizes (k per cycle) and tallies
    on both bank paths, in both Philox forms."""
    p = synth.two_zone_cubes(histories=50000, inactive=2, active=3)
    xml = p.xml()
    for fast in (0, 1):
        a = gpu_ctx(xml).run_keigenvalue(rng=RNG_PHILOX, fast_math=fast, bank_path=BANK_SLOTS)
        b = gpu_ctx(xml).run_keigenvalue(rng=RNG_PHILOX, fast_math=fast, bank_path=BANK_DIRECT)
        assert np.array_equal(a.bank_size, b.bank_size)
        assert np.array_equal(a.k_cycle, b.k_cycle)
        np.testing.assert_allclose(b.sum, a.sum, rtol=FP_RTOL)


def test_bank_direct_path_rejected_where_counts_are_unknown(built_library):
    """The direct path needs Philox streams and chi cdfs that end above every
    threshold drawn: reference streams are refused, and so is the FP64 form
    for a chi whose normalised cdf ends one ulp short of the largest uniform
    it draws (the automatic choice takes the slot path there)."""
    p = synth.two_zone_cubes(histories=2000, groups=4, inactive=1, active=1)
    ctx = gpu_ctx(p.xml())
    with pytest.raises(MCError, match="direct bank path"):
        ctx.run_keigenvalue(rng=RNG_MINSTD, bank_path=BANK_DIRECT)
    # chi (1, 4, 1, 1) / 7: the cdf ends at 1 - 2^-52, the FP64 form's
    # largest uniform (the FP32 form draws at most 1 - 2^-24)
    p.nuclides[0].chi = np.tile(np.array([1.0, 4.0, 1.0, 1.0])[:, None], (1, 4))
    ctx = gpu_ctx(p.xml())
    with pytest.raises(MCError, match="direct bank path"):
        ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=0, bank_path=BANK_DIRECT)
    a = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=1, bank_path=BANK_DIRECT)
    b = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=1, bank_path=BANK_SLOTS)
    assert np.array_equal(a.bank_size, b.bank_size)
    r = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=0)
    assert (np.asarray(r.bank_size) > 0).all()


@pytest.mark.parametrize("rng,fast", [(RNG_PHILOX, 1), (RNG_MINSTD, 0)])
def test_keig_cycles_equal_cycle_by_cycle(rng, fast, built_library):
    """mc_keig_cycles (one synchronisation for many cycles, bank sizes and k
    kept on the device, sources drawn from the bank in place) gives the
    cycle-by-cycle loop's k per cycle, bank sizes and tallies, with both
    stream kinds (Philox: direct bank path; minstd: slots)."""
    xml = synth.two_zone_cubes(histories=40_000, inactive=3, active=4).xml()
    a, b = gpu_ctx(xml), gpu_ctx(xml)
    for ctx in (a, b):
        ctx.keig_begin(rng=rng, fast_math=fast, variant=2)
    ka = [a.keig_cycle(False) for _ in range(3)] + [a.keig_cycle(True) for _ in range(4)]
    kb = list(b.keig_cycles(3, False)) + list(b.keig_cycles(4, True))
    assert ka == kb
    oa, ob = a.keig_status(), b.keig_status()
    assert oa.events == ob.events
    ra, rb = a.keig_end(), b.keig_end()
    assert ra.k_mean == rb.k_mean and ra.k_std == rb.k_std


def test_run_keigenvalue_uses_cycles_and_checkpoint(built_library, tmp_path):
    """The full-run call (inactive and active phases through mc_keig_cycles)
    equals the cycle-by-cycle loop; a checkpoint taken after cycles run in
    one call writes the pending source out and resumes to the same k."""
    xml = synth.two_zone_cubes(histories=30_000, inactive=2, active=3).xml()
    a = gpu_ctx(xml)
    r = a.run_keigenvalue(rng=RNG_PHILOX, fast_math=1, variant=2)
    b = gpu_ctx(xml)
    b.keig_begin(rng=RNG_PHILOX, fast_math=1, variant=2)
    kb = [b.keig_cycle(i >= 2) for i in range(5)]
    assert list(r.k_cycle) == kb
    c = gpu_ctx(xml)
    c.keig_begin(rng=RNG_PHILOX, fast_math=1, variant=2)
    c.keig_cycles(2, False)
    blob = c.keig_checkpoint()
    d = gpu_ctx(xml)
    d.keig_resume(blob)
    assert list(d.keig_cycles(3, True)) == kb[2:]


@pytest.mark.parametrize("multi", [False, True])
def test_source_dying_out_is_reported(multi, built_library):
    """A strongly subcritical medium (k_inf = 0.04, 50 histories per cycle:
    a cycle banks no site with probability ~e^-2) loses its fission source
    within a few cycles: the per-cycle call and the multi-cycle call both
    report it ("source died out"), without reading past the empty bank, and
    the context stays usable."""
    xml = synth.infinite_medium(c=0.25, capture=0.72, fission=0.03, nubar=1.0, histories=50, keig=(60, 0)).xml()
    ctx = gpu_ctx(xml)
    ctx.keig_begin(rng=RNG_PHILOX, fast_math=1, variant=2)
    with pytest.raises(MCError, match="died out"):
        if multi:
            ctx.keig_cycles(60, False)
        else:
            for _ in range(60):
                ctx.keig_cycle(False)
    ctx.keig_end()
    ctx.load_xml(synth.one_group_cube(histories=5000, inactive=1, active=2).xml())
    r = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=1, variant=2)
    assert (np.asarray(r.k_cycle) > 0.5).all()
