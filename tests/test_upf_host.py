"""UPF reader and the tabulated radial functions on the host (no GPU).

The test files are written by tests/golden/make_test_upf.py (a Si-like Z = 4
pseudopotential with l = 0, 1 projectors, identical numbers in the v1 and v2
layouts).  The product's tables (cubic Hermite on a 0.005 Bohr^-1 grid) are
checked against the oracle's quadrature at every q.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from addft_gb300 import psp as P
from addft_gb300 import upf
from oracle import pw

GOLD = Path(__file__).resolve().parent / "golden"
V1, V2 = GOLD / "si_test_v1.upf", GOLD / "si_test_v2.upf"


def test_v1_and_v2_layouts_parse_to_the_same_arrays():
    a, b = upf.read_upf(V2), upf.read_upf(V1)
    assert a["mesh"] == b["mesh"] == 1085 and list(a["lll"]) == list(b["lll"]) == [0, 1]
    for k in ("r", "rab", "vloc_at", "betar", "dion"):
        assert np.array_equal(a[k], b[k])
    o = pw.read_upf(V2)
    for k in ("r", "rab", "vloc_at", "betar", "dion"):
        assert np.array_equal(a[k], o[k])
    assert a["zval"] == o["zval"] == 4.0 and not a["nlcc"]


def test_from_upf_units_and_nlcc_rejection(tmp_path):
    p = P.from_upf(V2)
    assert p.kind == 1 and p.zval == 4.0 and p.proj_l == (0, 1) and p.nh == 4
    assert np.allclose(p.dion, np.diag([0.8, -0.3]))             # Ry -> Ha
    bad = tmp_path / "nlcc.upf"
    bad.write_text(V2.read_text().replace('core_correction="F"', 'core_correction="T"'))
    with pytest.raises(NotImplementedError):
        P.from_upf(bad)


def _hermite(tab, dq, f, q):
    x = q / dq
    i = np.minimum(x.astype(int), tab.shape[-1] - 2)
    s = x - i
    y0, y1, m0, m1 = tab[f, 0, i], tab[f, 0, i + 1], tab[f, 1, i] * dq, tab[f, 1, i + 1] * dq
    return (2 * s ** 3 - 3 * s ** 2 + 1) * y0 + (s ** 3 - 2 * s ** 2 + s) * m0 + (-2 * s ** 3 + 3 * s ** 2) * y1 \
        + (s ** 3 - s ** 2) * m1


def test_tables_match_oracle_quadrature():
    p, o = P.from_upf(V2), pw.from_upf(V1)
    tab, dq = p.host_table()
    q = np.concatenate([[0.0], np.random.default_rng(0).uniform(0.05, 25.0, 300)])
    beta = pw.beta_q(o, q)
    for f in range(2):
        assert np.max(np.abs(_hermite(tab, dq, f, q) - beta[f])) < 1e-9 * np.max(np.abs(beta[f]))
    qq = q[1:]
    coul = 4 * np.pi * 4.0 * np.exp(-qq ** 2 / 4) / qq ** 2
    v = pw.vloc_q(o, qq)
    assert np.max(np.abs(_hermite(tab, dq, 2, qq) - coul - v)) < 1e-9 * np.max(np.abs(v + coul))
    assert abs(p.vloc_g0() - float(pw.vloc_q(o, np.array([0.0]))[0])) < 1e-12


def test_unsupported_projectors_and_malformed_files_are_rejected(tmp_path):
    """An l = 3 projector reads, but building the device tables rejects it (the reference's
    real Y_lm and the GPU kernels go to l = 2); a v1 file without its header cannot be read."""
    d = tmp_path / "f.upf"
    d.write_text(V2.read_text().replace('index="2" angular_momentum="1"', 'index="2" angular_momentum="3"'))
    p = P.from_upf(d)
    assert p.proj_l == (0, 3) and p.nh == 8
    with pytest.raises(NotImplementedError, match="l > 2"):
        p.c_struct()
    h = tmp_path / "noheader.upf"
    text = V1.read_text()
    h.write_text(text[text.index("</PP_HEADER>") + len("</PP_HEADER>"):])
    with pytest.raises(ValueError, match="PP_HEADER"):
        P.from_upf(h)


def test_d_channel_tables_match_oracle_quadrature():
    """The l = 2 projector of tests/golden/si_test_d_v2.upf: the product's Hermite table of
    4 pi int r beta(r) r j_2(q r) dr against the oracle's quadrature at every q, and j_2
    itself against the closed form / series of the reference (psp.py:72-83)."""
    D = GOLD / "si_test_d_v2.upf"
    p, o = P.from_upf(D), pw.from_upf(D)
    assert p.proj_l == (0, 1, 2) and p.nh == 9
    tab, dq = p.host_table()
    q = np.concatenate([[0.0], np.random.default_rng(1).uniform(0.05, 25.0, 300)])
    beta = pw.beta_q(o, q)
    for f in range(3):
        assert np.max(np.abs(_hermite(tab, dq, f, q) - beta[f])) < 1e-9 * np.max(np.abs(beta[f]))
    x = np.linspace(0.0, 20.0, 2001)
    j2 = np.where(x > 0, (3 / np.where(x > 0, x, 1) ** 3 - 1 / np.where(x > 0, x, 1)) * np.sin(x)
                  - 3 * np.cos(x) / np.where(x > 0, x, 1) ** 2, 0.0)
    jp, _ = P._sph_j(2, x)
    jo, _ = pw._sph_jl(2, x)
    big = x > 0.5
    assert np.max(np.abs(jp[big] - j2[big])) < 1e-13 and np.max(np.abs(jo[big] - j2[big])) < 1e-13
    assert np.max(np.abs(jp - jo)) < 1e-13


def _arr_checks(x):
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    w = np.random.default_rng(11).normal(size=x.size)
    return {"size": int(x.size), "sum": float(np.sum(x)), "sumsq": float(np.sum(x * x)), "proj": float(x @ w),
            "head": x[:4].tolist(), "tail": x[-4:].tolist()}


@pytest.mark.parametrize("fname", ["si_test_v1.upf", "si_test_v2.upf", "si_test_d_v2.upf"])
def test_reader_and_radial_transforms_match_reference_code(fname):
    """Our UPF reader and the oracle's radial transforms against the reference's own
    geometry/upf.py read_upf and geometry/psp.py beta_q / vloc_q on the same files
    (tests/golden/make_reference_fixtures.py): every field (arrays by size, sum, sum of
    squares, a seeded projection and the end values) within 1e-13 relative, the transforms
    on a q grid within 1e-12 relative."""
    import json
    from pathlib import Path
    from oracle import pw
    gold = Path(__file__).resolve().parent / "golden"
    fix = json.loads((gold / "ref_fixtures.json").read_text())["upf_reader"]
    ref = fix["files"][fname]
    d = upf.read_upf(gold / fname)
    for k, v in ref.items():
        if k in ("beta_q", "vloc_q"):
            continue
        mine = d[k]
        if isinstance(v, dict):
            c = _arr_checks(mine)
            assert c["size"] == v["size"], k
            for key in ("sum", "sumsq", "proj"):
                assert abs(c[key] - v[key]) <= 1e-13 * max(1.0, abs(v[key])), (k, key)
            assert np.allclose(c["head"], v["head"], rtol=1e-14, atol=0) and np.allclose(c["tail"], v["tail"],
                                                                                          rtol=1e-14, atol=0), k
        else:
            assert np.array_equal(np.asarray(mine), np.asarray(v)), k
    q = np.asarray(fix["q"])
    psp = pw.from_upf(gold / fname)
    bq = np.asarray(pw.beta_q(psp, q))
    rb = np.asarray(ref["beta_q"])
    assert np.max(np.abs(bq - rb)) <= 1e-12 * np.max(np.abs(rb))
    vq = np.asarray(pw.vloc_q(psp, q[1:]))
    rv = np.asarray(ref["vloc_q"])
    assert np.max(np.abs(vq - rv)) <= 1e-12 * np.max(np.abs(rv))
