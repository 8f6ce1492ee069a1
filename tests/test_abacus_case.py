"""ABACUS case directories on the host: INPUT / KPT / STRU parsing and setup_from_case
(adapters/abacus/io.py).  The case uses the Si-like test UPF of tests/golden."""

from __future__ import annotations

import shutil
from pathlib import Path

import numpy as np
import pytest

import addft_gb300 as ad
from addft_gb300 import abacus

GOLD = Path(__file__).resolve().parent / "golden"


def _case(tmp_path, cart=False, kpt="K_POINTS\n0\nMonkhorst-Pack\n2 2 2 1 1 1\n", extra=""):
    (tmp_path / "pp").mkdir()
    shutil.copy(GOLD / "si_test_v2.upf", tmp_path / "pp" / "Si.upf")
    (tmp_path / "INPUT").write_text("INPUT_PARAMETERS\n# a comment\necutwfc 16   # Ry\nnbands 8\n"
                                    "pseudo_dir pp\nsmearing_method gaussian\nsmearing_sigma 0.02\n"
                                    "cal_force 1\ncal_stress 1\ncalculation scf\n" + extra)
    (tmp_path / "KPT").write_text(kpt)
    pos = ("Cartesian\nSi\n0.0\n2\n0.0 0.0 0.0 1 1 1\n0.25 0.25 0.25 1 1 1\n" if cart else
           "Direct\nSi\n0.0\n2\n0.0 0.0 0.0 1 1 1\n0.25 0.25 0.25 1 1 1\n")
    (tmp_path / "STRU").write_text("ATOMIC_SPECIES\nSi 28.085 Si.upf\n\nLATTICE_CONSTANT\n10.2\n\n"
                                   "LATTICE_VECTORS\n0.0 0.5 0.5\n0.5 0.0 0.5\n0.5 0.5 0.0\n\n"
                                   "ATOMIC_POSITIONS\n" + pos)
    return tmp_path


def test_input_units_and_errors(tmp_path):
    c = _case(tmp_path)
    inp = abacus.read_input(c / "INPUT")
    assert inp.setup_args == {"ecut": 8.0, "nband": 8, "sigma": 0.01}
    assert inp.tasks == {"smearing": "gaussian", "cal_force": True, "cal_stress": True, "calculation": "scf"}
    assert inp.files == {"pseudo_dir": "pp"}
    (tmp_path / "BAD").write_text("ecutwfc 10\nsome_new_key 3\n")
    with pytest.raises(abacus.UnmappedParameterError):
        abacus.read_input(tmp_path / "BAD")
    (tmp_path / "BAD2").write_text("ecutwfc 10\ndft_plus_u 1\n")
    with pytest.raises(abacus.UnmappedParameterError):
        abacus.read_input(tmp_path / "BAD2")


def test_kpt_and_stru(tmp_path):
    c = _case(tmp_path)
    assert abacus.read_kpt(c / "KPT") == {"mode": "mp", "mesh": (2, 2, 2), "shift": (0.5, 0.5, 0.5)}
    (tmp_path / "KG").write_text("K_POINTS\n0\nGamma\n1 1 1 0 0 0\n")
    assert abacus.read_kpt(tmp_path / "KG") == {"mode": "gamma"}
    s = abacus.read_stru(c / "STRU")
    assert np.allclose(s["lattice"], 10.2 * np.array([[0, .5, .5], [.5, 0, .5], [.5, .5, 0]]))
    assert np.allclose(s["frac"], [[0, 0, 0], [.25, .25, .25]]) and s["species"] == ["Si", "Si"]


def test_cartesian_positions_are_in_lattice_constant_units(tmp_path):
    s = abacus.read_stru(_case(tmp_path, cart=True) / "STRU")
    # Cartesian (0.25, 0.25, 0.25) lat0 is frac (0.25, 0.25, 0.25) in this fcc cell
    assert np.allclose(s["frac"][1], [0.25, 0.25, 0.25])


def test_setup_from_case_builds_the_system(tmp_path):
    sysm = ad.setup_from_case(_case(tmp_path))
    st = sysm.static
    assert st.natom == 2 and st.nband == 8 and st.psp.kind == 1 and st.psp.zval == 4.0
    assert st.nk == 8 and abs(st.sigma - 0.01) < 1e-15 and st.nelec == 8.0
    assert np.allclose(sysm.geo.lattice, 10.2 * np.array([[0, .5, .5], [.5, 0, .5], [.5, .5, 0]]))


def test_error_paths_are_loud(tmp_path):
    """Every unsupported or malformed input is an error, never a silent default
    (adapters/abacus/io.py:47-52, :112-206)."""
    c = _case(tmp_path)
    stru = (c / "STRU").read_text()
    (tmp_path / "S_unknown").write_text(stru.replace("ATOMIC_POSITIONS\nDirect\nSi", "ATOMIC_POSITIONS\nDirect\nGe"))
    with pytest.raises(ValueError, match="not in ATOMIC_SPECIES"):
        abacus.read_stru(tmp_path / "S_unknown")
    (tmp_path / "S_nopos").write_text(stru[:stru.index("ATOMIC_POSITIONS")])
    with pytest.raises(ValueError, match="without ATOMIC_POSITIONS"):
        abacus.read_stru(tmp_path / "S_nopos")
    (tmp_path / "S_mode").write_text(stru.replace("ATOMIC_POSITIONS\nDirect", "ATOMIC_POSITIONS\nCartesian_angstrom"))
    with pytest.raises(NotImplementedError):
        abacus.read_stru(tmp_path / "S_mode")
    (tmp_path / "I_spin").write_text("ecutwfc 10\nnspin 2\n")
    with pytest.raises(abacus.UnmappedParameterError, match="nspin"):
        abacus.read_input(tmp_path / "I_spin")
    (tmp_path / "I_noval").write_text("ecutwfc\n")
    with pytest.raises(abacus.UnmappedParameterError):
        abacus.read_input(tmp_path / "I_noval")
    (tmp_path / "KPT_empty").write_text("# nothing\n")
    with pytest.raises(ValueError):
        abacus.read_kpt(tmp_path / "KPT_empty")
    (tmp_path / "KPT_list").write_text("K_POINTS\n2\nDirect\n0 0 0 1\n0.5 0 0 1\n")
    with pytest.raises(NotImplementedError):
        abacus.read_kpt(tmp_path / "KPT_list")
    for bad in ("basis_type lcao", "dft_functional pbe", "ntype 2"):
        (tmp_path / "I_req").write_text("ecutwfc 10\n" + bad + "\n")
        with pytest.raises(abacus.UnmappedParameterError, match=bad.split()[0]):
            abacus.read_input(tmp_path / "I_req")
    (tmp_path / "S_short").write_text(stru.replace("0.25 0.25 0.25 1 1 1\n", ""))
    with pytest.raises(ValueError, match="ends inside"):
        abacus.read_stru(tmp_path / "S_short")


def test_case_without_ecut_or_with_two_species_is_rejected(tmp_path):
    c = _case(tmp_path)
    (c / "INPUT").write_text("INPUT_PARAMETERS\nnbands 8\npseudo_dir pp\n")
    with pytest.raises(abacus.UnmappedParameterError, match="ecutwfc"):
        ad.setup_from_case(c)
    (c / "INPUT").write_text("INPUT_PARAMETERS\necutwfc 16\nnbands 8\npseudo_dir pp\n")
    stru = (c / "STRU").read_text()
    two = stru.replace("Si 28.085 Si.upf\n", "Si 28.085 Si.upf\nC 12.011 Si.upf\n")
    two = two.replace("2\n0.0 0.0 0.0 1 1 1\n0.25 0.25 0.25 1 1 1\n",
                      "1\n0.0 0.0 0.0 1 1 1\nC\n0.0\n1\n0.25 0.25 0.25 1 1 1\n")
    (c / "STRU").write_text(two)
    assert abacus.read_stru(c / "STRU")["species"] == ["Si", "C"]
    with pytest.raises(NotImplementedError, match="one species"):
        ad.setup_from_case(c)


def test_scf_keywords_and_accepted_options_are_recorded(tmp_path):
    c = _case(tmp_path, extra="scf_thr 1e-9\nscf_nmax 80\nmixing_beta 0.4\nks_solver cg\nsymmetry 0\n")
    case = abacus.read_case(c)
    assert case.scf_args == {"tol": 1e-9, "max_iter": 80, "beta": 0.4}
    assert case.input.info == {"ks_solver": "cg", "symmetry": "0"}
    kw = case.setup_kwargs()
    assert kw["ecut"] == 8.0 and kw["nband"] == 8 and kw["sigma"] == 0.01


def test_fixed_smearing_gives_zero_width(tmp_path):
    c = _case(tmp_path, kpt="K_POINTS\n0\nGamma\n1 1 1 0 0 0\n")
    (c / "INPUT").write_text("INPUT_PARAMETERS\necutwfc 16\nnbands 8\npseudo_dir pp\nsmearing_method fixed\n")
    st = ad.setup_from_case(c).static
    assert st.sigma == 0.0 and st.nk == 1


def test_setup_from_case_matches_reference_adapter(tmp_path):
    """Our ABACUS adapter against the System the reference's own adapters/abacus/io.py builds
    from the same case directories (tests/golden/make_reference_fixtures.py): cell, basis,
    k points and weights, bands, smearing and electron count."""
    import json
    fix = json.loads((GOLD / "ref_fixtures.json").read_text())["abacus"]
    for i, (name, c) in enumerate(fix.items()):
        d = tmp_path / name
        d.mkdir()
        s = ad.setup_from_case(_case(d, **c["case"]))
        st = s.static
        assert np.allclose(s.geo.lattice, c["lattice"], rtol=0, atol=1e-12), name
        assert np.allclose(s.geo.frac, c["frac"], rtol=0, atol=1e-12), name
        assert st.basis.nG == c["nG"] and list(st.basis.fft_shape) == c["fft_shape"], name
        assert abs(st.basis.ecut - c["ecut"]) < 1e-12 and st.nband == c["nband"], name
        assert abs(st.sigma - c["sigma"]) < 1e-15 and abs(st.nelec - c["nelec"]) < 1e-12, name
        assert np.allclose(st.kpts, c["kpts"], rtol=0, atol=1e-12), name
        assert np.allclose(st.kweights, c["kweights"], rtol=0, atol=1e-14), name
