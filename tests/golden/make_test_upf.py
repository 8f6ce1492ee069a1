"""Writes the test pseudopotential files tests/golden/si_test_v2.upf,
si_test_v1.upf and si_test_d_v2.upf (with an added l = 2 projector): a Si-like (Z = 4) norm-conserving KB pseudopotential with one
l = 0 and one l = 1 projector, made from analytic shapes on a logarithmic
mesh (no real pseudopotential file is available offline).  Both files carry
the same numbers, in the UPF v2 (XML) and v1 (text) layouts.

  r_i = exp(-7 + 0.0125 i) / 14,  i < 1085      rab = 0.0125 r
  v_loc(r) = -2 Z erf(r / 1.0) / r + 1.6 exp(-(r / 0.9)^2)         (Ry)
  r beta_0(r) = 1.4 r^2 exp(-(r / 1.1)^2),  r beta_1(r) = 0.9 r^2 exp(-(r / 1.2)^2) r / 1.2
  D = diag(1.6, -0.6) Ry
"""

from math import erf
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def arrays():
    i = np.arange(1085)
    r = np.exp(-7.0 + 0.0125 * i) / 14.0
    rab = 0.0125 * r
    z = 4.0
    vloc = -2.0 * z * np.array([erf(x) for x in r / 1.0]) / r + 1.6 * np.exp(-(r / 0.9) ** 2)
    b0 = 1.4 * r ** 2 * np.exp(-(r / 1.1) ** 2)
    b1 = 0.9 * r ** 2 * np.exp(-(r / 1.2) ** 2) * r / 1.2
    return r, rab, vloc, np.stack([b0, b1]), np.diag([1.6, -0.6]), z


def fmt(a):
    return "\n".join(" ".join(f"{x: .14E}" for x in a[j:j + 4]) for j in range(0, len(a), 4))


def write():
    r, rab, vloc, betar, dion, z = arrays()
    n = r.size
    v2 = [f'<UPF version="2.0.1">', f'<PP_HEADER element="Si" pseudo_type="NC" z_valence="{z:.6f}" '
          f'core_correction="F" l_max="1" mesh_size="{n}" number_of_proj="2"/>',
          f'<PP_MESH><PP_R type="real" size="{n}">\n{fmt(r)}\n</PP_R>',
          f'<PP_RAB type="real" size="{n}">\n{fmt(rab)}\n</PP_RAB></PP_MESH>',
          f'<PP_LOCAL type="real" size="{n}">\n{fmt(vloc)}\n</PP_LOCAL>', '<PP_NONLOCAL>']
    for ib, l in enumerate((0, 1)):
        v2.append(f'<PP_BETA.{ib + 1} type="real" size="{n}" index="{ib + 1}" angular_momentum="{l}">\n'
                  f'{fmt(betar[ib])}\n</PP_BETA.{ib + 1}>')
    v2 += [f'<PP_DIJ type="real" size="4">\n{fmt(dion.reshape(-1))}\n</PP_DIJ>', '</PP_NONLOCAL>', '</UPF>']
    (HERE / "si_test_v2.upf").write_text("\n".join(v2) + "\n")
    v1 = ["<PP_HEADER>", "   0                   Version Number", "  Si                   Element",
          "   NC                  Norm - Conserving pseudopotential", "    F                  Nonlinear Core Correction",
          " SLA PZ NOGX NOGC   PZ   Exchange-Correlation functional",
          f"    {z:.8f}          Z valence", "    0.00000000000      Total energy",
          "    0.0000000    0.0000000 Suggested cutoff for wfc and rho", "    1                  Max angular momentum component",
          f"  {n}                 Number of points in mesh", "    0    2             Number of Wavefunctions, Number of Projectors",
          "</PP_HEADER>", "<PP_MESH>", f"<PP_R>\n{fmt(r)}\n</PP_R>", f"<PP_RAB>\n{fmt(rab)}\n</PP_RAB>", "</PP_MESH>",
          f"<PP_LOCAL>\n{fmt(vloc)}\n</PP_LOCAL>", "<PP_NONLOCAL>"]
    for ib, l in enumerate((0, 1)):
        v1.append(f"<PP_BETA>\n    {ib + 1}    {l}             Beta    L\n   {n}\n{fmt(betar[ib])}\n</PP_BETA>")
    v1 += ["<PP_DIJ>", "    2                  Number of nonzero Dij",
           f"    1    1  {dion[0, 0]: .14E}", f"    2    2  {dion[1, 1]: .14E}", "</PP_DIJ>", "</PP_NONLOCAL>"]
    (HERE / "si_test_v1.upf").write_text("\n".join(v1) + "\n")


def write_d():
    """si_test_d_v2.upf: the same file with a third, l = 2 projector
    r beta_2(r) = 0.7 r^3 exp(-(r / 1.0)^2) and D = diag(1.6, -0.6, 0.4) Ry (UPF v2)."""
    r, rab, vloc, betar, dion, z = arrays()
    b2 = 0.7 * r ** 3 * np.exp(-(r / 1.0) ** 2)
    betar = np.concatenate([betar, b2[None]])
    dion = np.diag([1.6, -0.6, 0.4])
    n = r.size
    v2 = [f'<UPF version="2.0.1">', f'<PP_HEADER element="Si" pseudo_type="NC" z_valence="{z:.6f}" '
          f'core_correction="F" l_max="2" mesh_size="{n}" number_of_proj="3"/>',
          f'<PP_MESH><PP_R type="real" size="{n}">\n{fmt(r)}\n</PP_R>',
          f'<PP_RAB type="real" size="{n}">\n{fmt(rab)}\n</PP_RAB></PP_MESH>',
          f'<PP_LOCAL type="real" size="{n}">\n{fmt(vloc)}\n</PP_LOCAL>', '<PP_NONLOCAL>']
    for ib, l in enumerate((0, 1, 2)):
        v2.append(f'<PP_BETA.{ib + 1} type="real" size="{n}" index="{ib + 1}" angular_momentum="{l}">\n'
                  f'{fmt(betar[ib])}\n</PP_BETA.{ib + 1}>')
    v2 += [f'<PP_DIJ type="real" size="9">\n{fmt(dion.reshape(-1))}\n</PP_DIJ>', '</PP_NONLOCAL>', '</UPF>']
    (HERE / "si_test_d_v2.upf").write_text("\n".join(v2) + "\n")


if __name__ == "__main__":
    write()
    write_d()
