"""The oracle against the reference's own code (CPU).

oracle/ref/build_ref.py compiles the reference's sources unmodified with
stand-ins for pugixml and the HDF5 C++ API; its Driver::Create(path)->Solve()
runs each problem, and the oracle (with the reference's geometry semantics)
must give the same estimator means on the same histories, seeds and
reference random streams, bit for bit.  This pins the oracle's multigroup,
continuous-energy, free-gas, delta-tracking and thermal-scattering
restatements on the reference itself.  Skipped where the reference checkout
is absent (the GPU machine).
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from minimc_gb300 import synth_ce, synth_tsl
from minimc_gb300.synth import with_sensitivities
from oracle.build import Oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def ref():
    try:
        from oracle.ref import build_ref
    except ImportError:
        pytest.skip("reference build recipe unavailable")
    lib_path = build_ref.build()
    if lib_path is None:
        pytest.skip("reference sources are not present")
    lib = C.CDLL(str(lib_path))
    lib.ref_solve.argtypes = [C.c_char_p, C.c_char_p, C.c_uint64, C.POINTER(C.c_double), C.c_char_p, C.c_size_t,
                              C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t]
    lib.ref_solve.restype = C.c_int
    lib.ref_keig.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, C.c_int, C.POINTER(C.c_double),
                             C.POINTER(C.c_uint64), C.c_char_p, C.c_uint64, C.POINTER(C.c_double),
                             C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_char_p, C.c_size_t, C.c_char_p,
                             C.c_size_t]
    lib.ref_keig.restype = C.c_int
    return lib


def align_orders(o: Oracle, orders: str):
    """The reference iterates a material's nuclides in the order of their
    heap addresses in its process (std::map keyed by shared_ptr), which need
    not be the order of creation; give the oracle the order the reference's
    run used for each material."""
    for cell, line in enumerate(orders.splitlines()):
        names = line.split("|", 1)[1].split()
        mat = o.cell_material(cell)
        if mat >= 0 and names:
            o.set_material_order(mat, names)


def absolute_paths(xml: str, d: Path) -> str:
    """The reference opens data files relative to the working directory."""
    return re.sub(r'="([^"/]+\.mctab)"', lambda m: f'="{d}/{m.group(1)}"', xml)


def run_both(ref, xml: str, d: Path, tmp_path: Path, estimator: str, quirks=True):
    n = int(re.search(r"<histories>(\d+)</histories>", xml).group(1))
    m = re.search(r"<seed>(\d+)</seed>", xml)
    seed = int(m.group(1)) if m else 1  # Driver: seed 1 when absent (src/Driver.cpp:41-44)
    o = Oracle(xml, d)
    o.set_quirks(quirks)
    path = tmp_path / "problem.xml"
    path.write_text(absolute_paths(xml, d))
    mean = np.zeros(max(1, o.total_bins))
    orders = C.create_string_buffer(1 << 16)
    text = C.create_string_buffer(1 << 22)
    err = C.create_string_buffer(2048)
    rc = ref.ref_solve(str(path).encode(), (estimator or "").encode(), len(mean), mean.ctypes.data_as(C.POINTER(C.c_double)),
                       orders, 1 << 16, text, 1 << 22, err, 2048)
    assert rc == 0, err.value.decode()
    align_orders(o, orders.value.decode())
    r = o.run_fixed_source(n, seed, threads=1)
    r["ref_text"] = text.value.decode()
    return r["sum"] / n, mean[: o.total_bins], r


def test_multigroup_fixtures(ref, tmp_path):
    for name, est in (("point_source_leakage.xml", "leakage"), ("mg_spheres.xml", None)):
        xml = (GOLDEN / name).read_text()
        if est is None:
            est = re.search(r'<current name="([^"]+)"', xml).group(1)
        got, want, _ = run_both(ref, xml, GOLDEN, tmp_path, est)
        assert np.array_equal(got[: len(want)], want), (name, got, want)


@pytest.fixture(scope="module")
def ce_files(tmp_path_factory):
    d = tmp_path_factory.mktemp("ce")
    return d, synth_ce.write_nuclides(d, n_grid=5000)


@pytest.mark.parametrize("temperature", [293.6, 600.0])
def test_continuous_energy_free_gas(ref, ce_files, tmp_path, temperature):
    d, files = ce_files
    xml = synth_ce.ce_problem_xml(files, histories=4000, keig=False, sphere=6.0, afrac=(0.6, 0.3, 0.001),
                                  temperature=temperature,
                                  estimators=[synth_ce.energy_current("leak", "sphere", bins=40)])
    got, want, r = run_both(ref, xml, d, tmp_path, "leak")
    assert r["secondaries"] > 0
    assert np.array_equal(got, want)


def test_delta_tracking_linear_temperature(ref, ce_files, tmp_path):
    d, files = ce_files
    temp = ("  <linear>\n    <gradient x=\"10.0\" y=\"0\" z=\"0\"/>\n    <intercept b=\"393.6\"/>\n"
            "    <bounds upper=\"493.6\" lower=\"293.6\"/>\n  </linear>")
    xml = synth_ce.ce_problem_xml(files, histories=2000, keig=False, sphere=6.0, afrac=(0.6, 0.3, 0.001),
                                  tracking="cell delta", temperature_xml=temp,
                                  estimators=[synth_ce.energy_current("leak", "sphere", bins=40)])
    got, want, _ = run_both(ref, xml, d, tmp_path, "leak")
    assert np.array_equal(got, want)


def test_thermal_scattering_broomstick(ref, tmp_path_factory, tmp_path):
    d = tmp_path_factory.mktemp("tsl")
    tsl = synth_tsl.write_tsl(d)
    nuc = synth_tsl.moderator_nuclide(d)
    xml = synth_tsl.broomstick_xml(tsl, nuc, histories=5000, energy=0.1e-6, temperature=450.0, cosine_bins=20,
                                   energy_bins=40)
    got, want, _ = run_both(ref, xml, d, tmp_path, "leakage")
    assert np.array_equal(got, want)


def test_continuous_temperature_delta_tracking_thermal(ref, tmp_path_factory, tmp_path):
    """The reference's continuous-temperature benchmark shape: cell delta
    tracking through a slab of the bound moderator whose flights are bounded
    by the thermal library's majorant (ThermalScattering::GetMajorant,
    src/ThermalScattering.cpp:106-109; CellDeltaTracking::Transport,
    src/TransportMethod.cpp:88-122), a linear temperature field 300-600 K,
    POD SampleBeta/SampleAlpha at every real thermal collision: the oracle's
    leakage means equal the reference's bit for bit."""
    d = tmp_path_factory.mktemp("tsl_ct")
    tsl = synth_tsl.write_tsl(d)
    nuc = synth_tsl.moderator_nuclide(d)
    xml = synth_tsl.continuous_temperature_slab_xml(tsl, nuc, histories=1500, thickness=1.0)
    got, want, r = run_both(ref, xml, d, tmp_path, "leakage")
    assert r["events"] > 3 * 1500  # real and virtual collisions happen
    assert np.array_equal(got, want)


def test_result_file_text(ref, ce_files, tmp_path, built_library):
    """The engine's result-file text (mc_output_format, the formatter behind
    Driver.write_output) for the oracle's tallies equals the reference's own
    .out text character for character: batch size line, logspace and
    linspace bin edges, 'none' bins, means and standard deviations."""
    from minimc_gb300.engine import format_output

    d, files = ce_files
    est = [synth_ce.energy_current("leak", "sphere", bins=40),
           '  <current name="plain" surface="sphere"/>',
           '  <current name="angle" surface="sphere">\n    <bins>\n      <cosine u="0" v="0" w="1">'
           '<linspace bins="7" min="-1" max="1"/></cosine>\n'
           '      <energy><boundaries>1e-6 1e-3 0.1 1.0</boundaries></energy>\n    </bins>\n  </current>']
    xml = synth_ce.ce_problem_xml(files, histories=3000, keig=False, sphere=6.0, afrac=(0.6, 0.3, 0.001),
                                  estimators=est)
    _, _, r = run_both(ref, xml, d, tmp_path, None)
    got = format_output(xml, d, r["sum"], r["sum_sq"], 3000)
    assert got == r["ref_text"]
    assert got.count("mean\n----\n") == 3


def test_result_file_text_multigroup(ref, tmp_path, built_library):
    from minimc_gb300.engine import format_output

    xml = (GOLDEN / "mg_spheres.xml").read_text()
    est = re.search(r'<current name="([^"]+)"', xml).group(1)
    n = int(re.search(r"<histories>(\d+)</histories>", xml).group(1))
    _, _, r = run_both(ref, xml, GOLDEN, tmp_path, est)
    assert format_output(xml, GOLDEN, r["sum"], r["sum_sq"], n) == r["ref_text"]


def check_sensitivity_text(ref, xml, d, tmp_path):
    from minimc_gb300.engine import format_output

    n = int(re.search(r"<histories>(\d+)</histories>", xml).group(1))
    _, _, r = run_both(ref, xml, d, tmp_path, None)
    text = r["ref_text"]
    assert "::" in text
    assert format_output(xml, d, r["sum"], r["sum_sq"], n) == text
    return r


def test_sensitivities_multigroup(ref, tmp_path, built_library):
    """Sensitivity estimators of a current estimator to total cross-section
    perturbations of two nuclides (src/Perturbation.cpp:68-78,
    src/Sensitivity.cpp:55-58): the oracle's scores give the reference's
    own result text."""
    xml = with_sensitivities((GOLDEN / "mg_spheres.xml").read_text(), [("dH", "hydrogen"), ("dO", "oxygen")])
    r = check_sensitivity_text(ref, xml, GOLDEN, tmp_path)
    # estimator bins, then one block per sensitivity
    assert len(r["sum"]) == 3 and r["sum"][1] != 0 and r["sum"][2] != 0


@pytest.mark.parametrize("tracking", ["surface", "cell delta"])
def test_sensitivities_continuous_energy(ref, ce_files, tmp_path, built_library, tracking):
    d, files = ce_files
    temp = None
    if tracking == "cell delta":
        temp = ("  <linear>\n    <gradient x=\"10.0\" y=\"0\" z=\"0\"/>\n    <intercept b=\"393.6\"/>\n"
                "    <bounds upper=\"493.6\" lower=\"293.6\"/>\n  </linear>")
    xml = synth_ce.ce_problem_xml(files, histories=2000, keig=False, sphere=6.0, afrac=(0.6, 0.3, 0.001),
                                  tracking=tracking, temperature_xml=temp,
                                  estimators=[synth_ce.energy_current("leak", "sphere", bins=20),
                                              '  <current name="plain" surface="sphere"/>'])
    xml = with_sensitivities(xml, [("dH1", "H1"), ("dU", "U235")])
    check_sensitivity_text(ref, xml, d, tmp_path)


@pytest.mark.parametrize("case", ["perturbation", "nuclide"])
def test_sensitivity_input_errors(tmp_path, built_library, case):
    """Unknown perturbation or nuclide names.  The reference forms these
    messages (src/Perturbation.cpp:98-118, src/World.cpp:63-81) inside
    noexcept constructors (src/Estimator.cpp:76-90, src/Perturbation.cpp:87-96),
    so its process terminates; here the load fails with the message."""
    from minimc_gb300.engine import MCError, format_output

    xml = with_sensitivities((GOLDEN / "mg_spheres.xml").read_text(), [("dH", "hydrogen")])
    if case == "perturbation":
        xml = xml.replace('<perturbation name="dH"/>', '<perturbation name="dX"/>')
        want = 'Perturbation "dX" not found. Must be one of: ["dH", ]'
    else:
        xml = xml.replace('nuclide="hydrogen"/>\n</perturbations>', 'nuclide="helium"/>\n</perturbations>')
        want = 'Nuclide "helium" not found. Must be one of: ['
    with pytest.raises(MCError) as e:
        format_output(xml, GOLDEN, [0.0] * 3, [0.0] * 3, 1)
    assert e.value.message.startswith(want), e.value.message


def run_keig_both(ref, xml: str, tmp_path: Path, estimator: str, nbins: int, inactive: int, active: int,
                  threads: int):
    """The reference's own transport in the k-eigenvalue loop (oracle/ref/
    harness.cpp: Particle::Transport per source particle, fission sites
    through Particle::MoveSecondariesTo, k = M/N, uniform resampling) and
    the oracle's loop on the same problem and seeds."""
    n = int(re.search(r"<histories>(\d+)</histories>", xml).group(1))
    o = Oracle(xml, tmp_path)
    o.set_quirks(True)
    path = tmp_path / "keig.xml"
    path.write_text(xml)
    cycles = inactive + active
    k = np.zeros(cycles)
    bank = np.zeros(cycles, np.uint64)
    mean = np.zeros(nbins)  # the named estimator's bins
    secs = C.c_double()
    lost = C.c_uint64()
    orders = C.create_string_buffer(1 << 16)
    err = C.create_string_buffer(2048)
    rc = ref.ref_keig(str(path).encode(), inactive, active, threads, k.ctypes.data_as(C.POINTER(C.c_double)),
                      bank.ctypes.data_as(C.POINTER(C.c_uint64)), estimator.encode(), len(mean),
                      mean.ctypes.data_as(C.POINTER(C.c_double)), C.byref(secs), C.byref(lost), orders, 1 << 16,
                      err, 2048)
    assert rc == 0, err.value.decode()
    align_orders(o, orders.value.decode())
    r = o.run_keigenvalue(n, 1, inactive, active, threads=threads)
    return {"k": k, "bank": bank, "mean": mean, "seconds": secs.value, "lost": lost.value}, r, n


@pytest.mark.parametrize("threads", [1, 4])
def test_keigenvalue_loop_on_reference_code(ref, tmp_path, threads):
    """k per cycle, bank sizes and (one thread: same summation order) the
    estimator means of the oracle's k-eigenvalue loop equal the reference's
    own transport run through the same loop, bit for bit: the one-group
    problem in a planex slab cut by a sphere, 5 inactive + 5 active cycles
    of 4,000 histories."""
    from minimc_gb300 import synth

    xml = synth.one_group_slab_sphere(histories=4000, inactive=5, active=5).xml()
    got, want, n = run_keig_both(ref, xml, tmp_path, "leak-ball", 1, 5, 5, threads)
    assert np.array_equal(got["bank"], want["bank_size"]), (got["bank"], want["bank_size"])
    assert np.array_equal(got["k"], want["k_cycle"])
    assert got["bank"].min() > 0
    if threads == 1:
        o_mean = want["sum"] / (n * 5)
        # leak-ball is the second of the oracle's flattened bins
        assert np.array_equal(got["mean"], o_mean[1:2])
    # fission sites banked beyond a surface a particle grazed without
    # crossing (the reference's fixed nudge) start in a void: lost in both
    assert got["lost"] == want["lost"]


def test_keigenvalue_two_zone_spheres_on_reference_code(ref, tmp_path):
    """The 8-group two-zone problem (same seeded data as the GPU benchmark)
    in concentric spheres: k per cycle and bank sizes of the oracle's loop
    equal the reference's own transport, and the group-binned leakage means
    too (one thread)."""
    from minimc_gb300 import synth

    xml = synth.two_zone_spheres(histories=3000, inactive=3, active=3).xml()
    got, want, n = run_keig_both(ref, xml, tmp_path, "leak", 10, 3, 3, 1)  # 8 groups + 2 open ends
    assert np.array_equal(got["bank"], want["bank_size"])
    assert np.array_equal(got["k"], want["k_cycle"])
    assert np.array_equal(got["mean"], want["sum"] / (n * 3))


def test_keigenvalue_thermal_group_rows_on_reference_code(ref, tmp_path):
    """The two-zone problem with thermal transfer rows in its two lowest
    groups (up- and downscatter between them and into group 6, as the
    batched workload's thermal groups make them) and a cell temperature:
    the oracle's k per cycle, bank sizes and leakage means equal the
    reference's own transport (Multigroup::Scatter samples the full
    column, src/Multigroup.cpp:249-265)."""
    from minimc_gb300 import synth, thermal_groups

    rows = np.random.default_rng(5).dirichlet(np.ones(8) * 0.5, size=2)
    rows[:, :5] = 0.0  # thermal scatters stay in groups 6-8
    base = synth.two_zone_spheres(histories=3000, inactive=3, active=3)
    xml = thermal_groups.with_thermal_rows(base, 451.5, rows).xml()
    assert 'temperature="451.5"' in xml
    got, want, n = run_keig_both(ref, xml, tmp_path, "leak", 10, 3, 3, 1)
    assert np.array_equal(got["bank"], want["bank_size"])
    assert np.array_equal(got["k"], want["k_cycle"])
    assert np.array_equal(got["mean"], want["sum"] / (n * 3))
