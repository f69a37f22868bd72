"""Checkpoint / resume of k-eigenvalue cycles through the C ABI: a run
stopped after any cycle and resumed, in a fresh context holding the same
problem, gives k per cycle and bank sizes identical to a run that did not
stop, and the same tallies up to the order of their floating-point atomic
sums (both random stream families, multigroup and continuous energy)."""
import numpy as np
import pytest

from minimc_gb300 import RNG_MINSTD, RNG_PHILOX, Context, MCError, synth, synth_ce

pytestmark = pytest.mark.gpu


def straight_and_resumed(xml, base, stop, rng, **kw):
    a = Context(0)
    a.load_xml(xml, base)
    ref = a.run_keigenvalue(rng=rng, **kw)
    ncyc = ref.inactive + ref.active
    b = Context(0)
    b.load_xml(xml, base)
    b.keig_begin(rng=rng, **kw)
    for c in range(stop):
        b.keig_cycle(c >= ref.inactive)
    state = b.keig_checkpoint()
    del b
    c2 = Context(0)
    c2.load_xml(xml, base)
    c2.keig_resume(state)
    for c in range(stop, ncyc):
        c2.keig_cycle(c >= ref.inactive)
    k = np.zeros(ncyc)
    bank = np.zeros(ncyc, np.uint64)
    s, q = np.zeros(max(1, c2.info.total_bins)), np.zeros(max(1, c2.info.total_bins))
    from minimc_gb300.engine import KeigOut, _dptr
    import ctypes as C
    out = KeigOut()
    out.k_cycle = _dptr(k)
    out.bank_size = bank.ctypes.data_as(C.POINTER(C.c_uint64))
    out.sum = _dptr(s)
    out.sum_sq = _dptr(q)
    c2.check(c2.lib.mc_keig_end(c2.h, C.byref(out)))
    return ref, k, bank, s[: c2.info.total_bins], q[: c2.info.total_bins], out


@pytest.mark.parametrize("rng", [RNG_PHILOX, RNG_MINSTD])
@pytest.mark.parametrize("stop", [3, 9])  # inside the inactive, then the active cycles
def test_multigroup_resume_identical(rng, stop, built_library):
    p = synth.two_zone_cubes(histories=20000, inactive=5, active=10, groups=4)
    ref, k, bank, s, q, out = straight_and_resumed(p.xml(), None, stop, rng)
    assert np.array_equal(k, ref.k_cycle)
    assert np.array_equal(bank, ref.bank_size)
    np.testing.assert_allclose(s, ref.sum, rtol=1e-12)
    np.testing.assert_allclose(q, ref.sum_sq, rtol=1e-12)
    assert out.k_mean == ref.k_mean and out.events == ref.raw.events


def test_continuous_energy_resume_identical(built_library, tmp_path):
    files = synth_ce.write_nuclides(tmp_path, n_grid=5000)
    xml = synth_ce.ce_problem_xml(files, histories=20000, inactive=3, active=5, half=20.0)
    ref, k, bank, s, q, _ = straight_and_resumed(xml, tmp_path, 4, RNG_PHILOX)
    assert np.array_equal(k, ref.k_cycle)
    np.testing.assert_allclose(s, ref.sum, rtol=1e-12)


def test_checkpoint_file_driver(built_library, tmp_path):
    """run_keigenvalue_checkpointed: a run interrupted (here: a fresh
    context) picks up from the last file written."""
    p = synth.two_zone_cubes(histories=10000, inactive=4, active=6, groups=4)
    xml = p.xml()
    a = Context(0)
    a.load_xml(xml)
    ref = a.run_keigenvalue(rng=RNG_PHILOX)
    path = tmp_path / "run.ckpt"
    b = Context(0)
    b.load_xml(xml)
    b.keig_begin(rng=RNG_PHILOX)
    for c in range(6):
        b.keig_cycle(c >= 4)
    path.write_bytes(b.keig_checkpoint())
    c2 = Context(0)
    c2.load_xml(xml)
    r = c2.run_keigenvalue_checkpointed(path, every=2, rng=RNG_PHILOX)
    assert np.array_equal(r.k_cycle, ref.k_cycle)
    np.testing.assert_allclose(r.sum, ref.sum, rtol=1e-12)


def test_resume_rejects_other_problem(built_library):
    a = Context(0)
    a.load_xml(synth.two_zone_cubes(histories=1000, inactive=1, active=1, groups=4).xml())
    a.keig_begin(rng=RNG_PHILOX)
    a.keig_cycle(False)
    state = a.keig_checkpoint()
    b = Context(0)
    b.load_xml(synth.one_group_cube(histories=1000, inactive=1, active=1).xml())
    with pytest.raises(MCError) as e:
        b.keig_resume(state)
    assert "another problem" in e.value.message
    with pytest.raises(MCError):
        b.keig_resume(state[:-8])
