"""The C-ABI library loads and exports every symbol include/gbode.h declares.
No compute calls: these run without a GPU."""
from __future__ import annotations

import os
import re
import subprocess

import pytest

from conftest import ROOT


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "gbode.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set()
    for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt):
        name = m.group(1)
        if name.startswith(("d", "gbode")) and not name.startswith(("dReal", "dNearCallback")):
            names.add(name)
    return names - {"defined"}


@pytest.fixture(scope="module")
def lib_path():
    from ode_gb300 import build
    return build.build()


def test_every_declared_symbol_is_exported(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = sorted(header_symbols() - exported)
    assert not missing, missing


def test_ctypes_prototypes_cover_header(lib_path):
    from ode_gb300 import ode
    assert header_symbols() <= set(ode.exported_names())
    L = ode.load(lib_path)
    assert L.dTestRand() == 1


def test_mass_helpers_match_reference_formulas(lib_path):
    """mass.cpp:118-210 without any device work."""
    import ctypes
    from ode_gb300 import ode
    L = ode.load(lib_path)
    m = ode.dMass()
    L.dMassSetBox(ctypes.byref(m), 2.0, 1.0, 2.0, 3.0)
    assert abs(m.mass - 12.0) < 1e-6
    assert abs(m.I[0] - 12.0 / 12 * (4 + 9)) < 1e-5
    L.dMassSetSphere(ctypes.byref(m), 1.0, 0.5)
    assert abs(m.mass - 4 / 3 * 3.14159265 * 0.125) < 1e-5


def test_rand_known_answers(lib_path):
    """misc.cpp:64-74: the reference's LCG golden outputs."""
    from ode_gb300 import ode
    L = ode.load(lib_path)
    L.dRandSetSeed(0)
    assert [L.dRand() for _ in range(5)] == [0x3c6ef35f, 0x47502932, 0xd1ccf6e9, 0xaaf95334, 0x6252e503]


C_PROGRAM = r"""
#include <stdio.h>
#include "gbode.h"
int main(void) {
    dInitODE2(0);
    dWorldID w = dWorldCreate();
    dBodyID a = dBodyCreate(w), b = dBodyCreate(w);
    dBodySetPosition(a, 0, -1, 0);
    dBodySetPosition(b, 0, 1, 0);
    dMass m;
    dMassSetBox(&m, 2.0f, 1.0f, 2.0f, 3.0f);
    dBodySetMass(a, &m);
    dJointID j = dJointCreateHinge(w, 0);
    dJointAttach(j, a, b);
    dJointSetHingeAnchor(j, 0, 0, 0);
    dJointSetHingeAxis(j, 1, 0, 0);
    dMatrix3 R;
    dRFromAxisAndAngle(R, 1, 0, 0, 0.23f);
    dBodySetRotation(a, R);
    printf("%.5f %.3f %d\n", (double)dJointGetHingeAngle(j), (double)m.mass, dAreConnected(a, b));
    dWorldDestroy(w);
    dCloseODE();
    return 0;
}
"""


@pytest.mark.parametrize("compiler,std", [("gcc", "-std=c99"), ("g++", "-std=c++17")])
def test_header_builds_a_c_program(lib_path, tmp_path, compiler, std):
    """An ODE-style C program compiles against include/gbode.h as strict C99
    and as C++17 (no warnings with -Wall -Wextra -pedantic), links -lgbode and
    runs its host-side calls (no GPU work: world, bodies, mass, hinge
    geometry)."""
    src = tmp_path / "prog.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "prog"
    libdir = os.path.dirname(lib_path)
    lang = ["-x", "c++"] if compiler == "g++" else []
    cc = subprocess.run([compiler, std, "-Wall", "-Wextra", "-pedantic", "-Werror", *lang,
                         f"-I{os.path.join(ROOT, 'include')}", str(src), f"-L{libdir}", "-lgbode",
                         f"-Wl,-rpath,{libdir}", "-lm", "-o", str(exe)], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    angle, mass, connected = out.stdout.split()
    assert abs(float(angle) - 0.23) < 1e-4 and abs(float(mass) - 12.0) < 1e-3 and connected == "1"


@pytest.mark.parametrize("direction", [1, 2, 3])
def test_capsule_mass_matches_reference_formula(lib_path, direction):
    """mass.cpp:141-162 dMassSetCapsule: cylinder plus the two caps, the
    inertia about the capsule's axis on `direction`, the other two equal."""
    import ctypes
    import math
    from ode_gb300 import ode
    L = ode.load(lib_path)
    m = ode.dMass()
    rho, r, length = 700.0, 0.05, 0.3
    L.dMassSetCapsule(ctypes.byref(m), rho, direction, r, length)
    m1 = math.pi * r * r * length * rho
    m2 = 4.0 / 3.0 * math.pi * r ** 3 * rho
    ia = m1 * (0.25 * r * r + length * length / 12.0) + m2 * (0.4 * r * r + 0.375 * r * length + 0.25 * length ** 2)
    ib = (0.5 * m1 + 0.4 * m2) * r * r
    assert abs(m.mass - (m1 + m2)) <= 1e-5 * (m1 + m2)
    diag = [m.I[0], m.I[5], m.I[10]]
    for k in range(3):
        want = ib if k == direction - 1 else ia
        assert abs(diag[k] - want) <= 1e-5 * want
    assert m.I[1] == m.I[2] == m.I[4] == m.I[6] == m.I[8] == m.I[9] == 0.0


def test_total_mass_variants(lib_path):
    """mass.cpp dMassSetSphereTotal / dMassSetBoxTotal: the density form
    rescaled to the given total (dMassAdjust), so the inertia scales with it:
    sphere I = 2/5 m r^2, box I = m (b^2 + c^2) / 12."""
    import ctypes
    from ode_gb300 import ode
    L = ode.load(lib_path)
    m = ode.dMass()
    L.dMassSetSphereTotal(ctypes.byref(m), 3.0, 0.5)
    assert abs(m.mass - 3.0) < 1e-6 and abs(m.I[0] - 0.4 * 3.0 * 0.25) < 1e-6
    L.dMassSetBoxTotal(ctypes.byref(m), 6.0, 1.0, 2.0, 3.0)
    assert abs(m.mass - 6.0) < 1e-6
    assert abs(m.I[0] - 6.0 * (4 + 9) / 12) < 1e-5 and abs(m.I[5] - 6.0 * (1 + 9) / 12) < 1e-5
    assert abs(m.I[10] - 6.0 * (1 + 4) / 12) < 1e-5
    L.dMassSetZero(ctypes.byref(m))
    assert m.mass == 0.0 and all(x == 0.0 for x in m.I)
