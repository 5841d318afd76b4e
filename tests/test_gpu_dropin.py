"""The drop-in layer (prototypes.h entry points, libcubens_dropin.so) against
the reference: each call replays an element, geometry or solver call whose
inputs and outputs the golden fixtures recorded from the reference's own
routines (tests/golden/make_golden.py), with the arrays in the reference's
layout. quad, test and dot are checked against the oracle.

Tolerances: 1e-12 relative for element quantities, 1e-9 for pivots and
1e-8 for solutions (as the element tests of the resident API).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from cubens import models
from dropin import loader

pytestmark = pytest.mark.gpu


def P(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1e-300, np.max(np.abs(b)))


def _lines(text):
    return text.splitlines()


def _mcode_from_jcode(jcode, conn, dofs):
    """mcode of elements with the given joint incidences (0-based) and DOF
    count per joint, from jcode (model.c:1007-1032 for trusses and shells)."""
    out = []
    for e in conn:
        for j in e:
            out += [jcode[j * 7 + d] for d in range(dofs)]
    return np.array(out, dtype=np.int64)


def _split3(c, ne):
    """triads (rows x^, y^, z^ per element) -> the reference's c1, c2, c3 arrays"""
    c = np.asarray(c).reshape(ne, 3, 3)
    return [np.ascontiguousarray(c[:, r, :].reshape(-1)) for r in range(3)]


class Shells:
    def __init__(self, golden_dir):
        z = np.load(golden_dir / "elem_shell_panel8.npz")
        self.z = z
        text = str(z["model_def"])
        self.o = oracle.OracleModel(text)
        o = self.o
        E, NJ = o.ne_sh, o.nj
        ln = _lines(text)
        self.conn = [tuple(int(v) - 1 for v in ln[6 + e].split(",")) for e in range(E)]
        self.minc = np.array([v + 1 for e in self.conn for v in e], dtype=np.int64)
        self.mcode = _mcode_from_jcode(o.jcode, self.conn, 6)
        self.emod = np.full(E, models.PANEL_E)
        self.nu = np.full(E, models.PANEL_NU)
        self.thick = np.full(E, models.PANEL_T)
        c0, self.farea = o.shell_initial()
        self.xlocal, self.slength = o.shell_geometry0()
        self.jcode = np.ascontiguousarray(o.jcode, dtype=np.int64)


@pytest.fixture(scope="module")
def libs():
    return loader.load()


def test_updatc_forces_sh_stiff_sh_match_reference(libs, golden_dir):
    g, d = libs
    s = Shells(golden_dir)
    z, o = s.z, s.o
    E, NJ, N = o.ne_sh, o.nj, o.neq
    g.cbg_set(NJ, 0, 0, E, N, 2, 3, 0.0)
    # updatc on the state before the increment
    x = np.array(z["x_before"])
    x_ip = np.zeros(3 * NJ)
    dd = np.ascontiguousarray(z["dd"])
    defl, area, slen = np.zeros(1), np.zeros(E), np.zeros(3 * E)
    c1, c2, c3 = np.zeros(3 * E), np.zeros(3 * E), np.zeros(3 * E)
    z1 = np.zeros(6)
    osf = np.zeros(1, dtype=np.int32)
    d.updatc(P(x), P(x_ip), P(z1), P(dd), P(defl), P(area), P(slen), P(z1), P(osf), P(z1), P(c1), P(c2), P(c3),
             P(s.minc), P(s.jcode))
    np.testing.assert_allclose(x, z["x_after"], rtol=0, atol=1e-12 * np.abs(z["x_after"]).max())
    np.testing.assert_array_equal(x_ip, z["x_before"])
    ci = np.stack([c1.reshape(E, 3), c2.reshape(E, 3), c3.reshape(E, 3)], axis=1).reshape(-1)
    assert _rel(ci, z["c_i"]) < 1e-13
    assert _rel(area, z["area_i"]) < 1e-13
    # forces_sh from the previous-iteration state
    cp1, cp2, cp3 = _split3(z["c_ip"], E)
    ef_ip = np.ascontiguousarray(z["ef_ip"])
    ef_i = np.zeros(18 * E)
    f = np.zeros(N)
    zero = np.zeros(18 * E)
    rc = d.forces_sh(P(f), P(ef_ip), P(ef_i), P(zero), P(zero), P(dd), P(np.zeros(N)), P(zero), P(x),
                     P(x_ip), P(s.emod), P(s.nu), P(s.xlocal), P(s.thick), P(s.farea), P(area), P(s.slength),
                     P(slen), P(np.zeros(E)), P(cp1), P(cp2), P(cp3), P(c1), P(c2), P(c3), P(s.minc),
                     P(s.mcode), P(s.jcode))
    assert rc == 0
    assert _rel(ef_i, z["ef_i"]) < 1e-12
    assert _rel(f, z["f"]) < 1e-12
    # forces accumulate into f_temp (the caller zeroes it, main.c:2781)
    f2 = np.ones(N)
    d.forces_sh(P(f2), P(ef_ip), P(ef_i), P(zero), P(zero), P(dd), P(np.zeros(N)), P(zero), P(x), P(x_ip),
                P(s.emod), P(s.nu), P(s.xlocal), P(s.thick), P(s.farea), P(area), P(s.slength), P(slen),
                P(np.zeros(E)), P(cp1), P(cp2), P(cp3), P(c1), P(c2), P(c3), P(s.minc), P(s.mcode),
                P(s.jcode))
    np.testing.assert_allclose(f2, 1.0 + f, rtol=1e-12, atol=1e-12 * np.abs(f).max())
    # stiff_sh of the state after the increment, into the skyline
    maxa = np.ascontiguousarray(z["maxa"], dtype=np.int64)
    ss = np.zeros(len(z["ss"]))
    d.stiff_sh(P(ss), P(s.emod), P(s.nu), P(x), P(s.xlocal), P(s.thick), P(s.farea), P(area), P(s.slength),
               P(slen), P(np.zeros(E)), P(c1), P(c2), P(c3), P(ef_i), P(np.zeros(N)), P(zero), P(zero), P(zero),
               P(maxa), P(s.minc), P(s.mcode))
    assert _rel(ss, z["ss"]) < 1e-12


def test_skyfact_skysolve_solve_match_reference(libs, golden_dir):
    g, d = libs
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    o = oracle.OracleModel(str(z["model_def"]))
    N = o.neq
    g.cbg_set(o.nj, 0, 0, o.ne_sh, N, 2, 3, 0.0)
    maxa = np.ascontiguousarray(z["maxa"], dtype=np.int64)
    ss = np.array(z["ss"])
    ssd = np.zeros(N)
    det = np.zeros(1, dtype=np.int32)
    rhs = np.array(o.q)
    assert d.skyfact(P(maxa), P(ss), P(ssd), P(rhs), 0, P(det)) == 0
    assert int(det[0]) == int(z["det"])
    assert _rel(ssd, z["ssd"]) < 1e-9
    assert d.skysolve(P(maxa), P(ss), P(ssd), P(rhs), 0, P(det)) == 0
    assert _rel(rhs, z["ldlt_solution"]) < 1e-8
    # the factored skyline goes back into ss: a solve from it alone (fact = 1, a
    # fresh copy so the cached device factor is not used) gives the same answer
    ss2 = ss.copy()
    rhs2 = np.array(o.q)
    assert d.skysolve(P(maxa), P(ss2), P(ssd), P(rhs2), 1, P(det)) == 0
    assert _rel(rhs2, z["ldlt_solution"]) < 1e-8
    # solve (ALGFLAG 3, solve.c:83-90): dd = r, factor, solve
    ss3 = np.array(z["ss"])
    dd = np.zeros(N)
    nul = None
    ssd3 = np.zeros(N)
    rc = d.solve(nul, P(ss3), nul, nul, nul, nul, P(np.array(o.q)), P(dd), P(maxa), P(ssd3), P(det), nul, nul,
                 nul, nul, nul, nul, nul, nul, nul, nul, nul, nul, nul, nul, C.c_double(0), C.c_double(0), nul, 0,
                 C.c_double(1), nul, nul, nul, nul, nul, 0)
    assert rc == 0
    assert _rel(dd, z["ldlt_solution"]) < 1e-8


def test_solve_newmark_effective_system(libs, golden_dir):
    g, d = libs
    z = np.load(golden_dir / "elem_frame_2x2x3.npz")
    o = oracle.OracleModel(str(z["model_def"]))
    N = o.neq
    dtv = 0.005
    g.cbg_set(o.nj, 0, o.ne_fr, 0, N, 2, 5, dtv)
    maxa = np.ascontiguousarray(z["maxa"], dtype=np.int64)
    ss = np.array(z["ss"])
    sm = np.array(z["sm"])
    rng = np.random.default_rng(3)
    r, vm, am = rng.normal(size=N), rng.normal(size=N), rng.normal(size=N)
    alpham, alphaf, ddt = 0.0, 0.0, 1.0
    lss = len(ss)
    keff, reff = np.zeros(lss), np.zeros(N)
    dd, ssd = np.zeros(N), np.zeros(N)
    det = np.zeros(1, dtype=np.int32)
    nul = None
    rc = d.solve(nul, P(ss), nul, P(sm), nul, nul, P(r), P(dd), P(maxa), P(ssd), P(det), P(np.zeros(N)), P(vm),
                 P(am), nul, nul, nul, nul, nul, P(keff), P(reff), nul, nul, nul, nul, C.c_double(alpham),
                 C.c_double(alphaf), nul, 0, C.c_double(ddt), nul, nul, nul, nul, nul, 0)
    assert rc == 0
    alpha = (1 - alpham + alphaf) ** 2 / 4
    a0, a2, a3 = 1 / (alpha * dtv ** 2), 1 / (alpha * dtv), 1 / (2 * alpha) - 1
    K = oracle.skyline_to_dense(maxa, np.array(z["ss"]), N)
    K[np.diag_indices(N)] += a0 * (1 - alpham) * sm / (1 - alphaf)
    R = r + sm * ((1 - alpham) * (vm * a2 + am * a3) - alpham * am) / (1 - alphaf)
    ref = np.linalg.solve(K, R)
    assert _rel(dd, ref) < 1e-8


def test_truss_entry_points_match_reference(libs, golden_dir):
    g, d = libs
    z = np.load(golden_dir / "elem_truss_c1.npz")
    text = str(z["model_def"])
    o = oracle.OracleModel(text)
    T, NJ, N = o.ne_tr, o.nj, o.neq
    g.cbg_set(NJ, T, 0, 0, N, 2, 3, 0.0)
    ln = _lines(text)
    conn = [tuple(int(v) - 1 for v in ln[6 + e].split(",")) for e in range(T)]
    mcode = _mcode_from_jcode(o.jcode, conn, 3)
    head = 6 + T
    ncons = ln[head:].index("0,0") + 1
    x0 = np.array([[float(v) for v in l.split(",")] for l in ln[head + ncons:head + ncons + NJ]])
    llen = np.array([np.linalg.norm(x0[b] - x0[a]) for a, b in conn])
    emod, area = np.full(T, 200e9), np.full(T, 1.0e-3)
    L_i = np.array(z["length_i"])
    dr = np.array(z["dir_i"]).reshape(T, 3)
    c1, c2, c3 = [np.ascontiguousarray(dr[:, k]) for k in range(3)]
    f = np.zeros(N)
    ef = np.zeros(2 * T)
    d.forces_tr(P(f), P(ef), P(np.zeros(N)), P(emod), P(area), P(llen), P(L_i), P(np.zeros(T)), P(c1), P(c2),
                P(c3), P(mcode))
    assert _rel(ef, z["ef_i"]) < 1e-12
    assert _rel(f, z["f"]) < 1e-12
    maxa = np.ascontiguousarray(z["maxa"], dtype=np.int64)
    ss = np.zeros(len(z["ss"]))
    d.stiff_tr(P(ss), P(emod), P(area), P(llen), P(L_i), P(np.zeros(T)), P(c1), P(c2), P(c3), P(ef), P(maxa),
               P(mcode))
    assert _rel(ss, z["ss"]) < 1e-12


def test_frame_entry_points_match_reference(libs, golden_dir):
    g, d = libs
    z = np.load(golden_dir / "elem_frame_2x2x3.npz")
    text = str(z["model_def"])
    o = oracle.OracleModel(text)
    F, NJ, N = o.ne_fr, o.nj, o.neq
    g.cbg_set(NJ, 0, F, 0, N, 2, 3, 0.0)
    ln = _lines(text)
    conn = [tuple(int(v) - 1 for v in ln[6 + e].split(",")) for e in range(F)]
    minc = np.array([v + 1 for e in conn for v in e], dtype=np.int64)
    head = 6 + F
    ncons = ln[head:].index("0,0") + 1
    k0 = head + ncons + NJ
    props = np.array([[float(v) for v in ln[k0 + e].split(",")] for e in range(F)])
    emod, gmod, dens, area, istr, iweak, ipol, iwarp = [np.ascontiguousarray(props[:, k]) for k in range(8)]
    aux = np.array([[float(v) for v in ln[k0 + F + 1 + e].split(",")] for e in range(F)]).reshape(-1)
    mcode = np.ascontiguousarray(o.frame_mcode(), dtype=np.int64)
    jcode = np.ascontiguousarray(o.jcode, dtype=np.int64)
    osf = np.zeros(F, dtype=np.int32)
    off = np.zeros(6 * F)
    rel = np.zeros(5 * F, dtype=np.int32)
    zf = np.zeros(14 * F)
    yl = np.zeros(2 * F, dtype=np.int32)
    # updatc: frame lengths and triads
    x = np.array(z["x_before"])
    x_ip = np.zeros(3 * NJ)
    xfr = np.zeros(6 * F)
    L_i = np.zeros(F)
    c1, c2, c3 = np.zeros(3 * F), np.zeros(3 * F), np.zeros(3 * F)
    d.updatc(P(x), P(x_ip), P(xfr), P(np.ascontiguousarray(z["dd"])), P(L_i), P(np.zeros(1)), P(np.zeros(1)),
             P(off), P(osf), P(aux), P(c1), P(c2), P(c3), P(minc), P(jcode))
    np.testing.assert_allclose(x, z["x_after"], rtol=0, atol=1e-14 * np.abs(z["x_after"]).max())
    ci = np.stack([c1.reshape(F, 3), c2.reshape(F, 3), c3.reshape(F, 3)], axis=1).reshape(-1)
    assert _rel(ci, z["c_i"]) < 1e-13
    assert _rel(L_i, z["len_i"]) < 1e-14
    # forces_fr
    cp1, cp2, cp3 = _split3(z["c_ip"], F)
    f = np.zeros(N)
    ef_i = np.zeros(14 * F)
    rc = d.forces_fr(P(f), P(np.ascontiguousarray(z["ef_ip"])), P(ef_i), P(zf), P(zf), P(zf.copy()), P(yl),
                     P(np.ascontiguousarray(z["dd"])), P(emod), P(gmod), P(area), P(off), P(osf),
                     P(np.ascontiguousarray(z["lref"])), P(np.ascontiguousarray(z["len_ip"])), P(istr), P(iweak),
                     P(ipol), P(iwarp), P(np.zeros(F)), P(np.zeros(F)), P(np.zeros(F)), P(cp1), P(cp2), P(cp3),
                     P(c1), P(c2), P(c3), P(rel), P(mcode), P(np.zeros(1)), P(np.zeros(1, dtype=np.int32)))
    assert rc == 0
    assert _rel(ef_i, z["ef_i"]) < 1e-12
    assert _rel(f, z["f"]) < 1e-12
    # stiff_fr of the new state
    maxa = np.ascontiguousarray(z["maxa"], dtype=np.int64)
    ss = np.zeros(len(z["ss"]))
    d.stiff_fr(P(ss), P(emod), P(gmod), P(area), P(off), P(osf), P(np.ascontiguousarray(z["lref"])), P(L_i),
               P(istr), P(iweak), P(ipol), P(iwarp), P(yl), P(np.zeros(F)), P(np.zeros(F)), P(np.zeros(F)), P(c1),
               P(c2), P(c3), P(ef_i), P(zf), P(rel), P(maxa), P(mcode))
    assert _rel(ss, z["ss"]) < 1e-12
    # mass_fr at the new coordinates: masses and the rewritten lengths
    sm = np.zeros(N)
    llen = np.array(z["lref"])
    d.mass_fr(P(sm), P(area), P(llen), P(istr), P(iweak), P(ipol), P(iwarp), P(dens), P(osf), P(off), P(x),
              P(xfr), P(minc), P(mcode), P(np.zeros(1)))
    assert _rel(sm, z["sm"]) < 1e-14
    assert _rel(llen, z["mass_len"]) < 1e-14


def test_quad_test_dot_match_oracle(libs):
    g, d = libs
    rng = np.random.default_rng(17)
    N = 5000
    g.cbg_set(1, 0, 0, 0, N, 2, 3, 0.0)
    dt, dp, ddr, ddq = (rng.normal(size=N) for _ in range(4))
    a, b, c = 2.0, 0.5, -1.0
    rc_o, dt_o, dd_o, dl_o, lp_o = oracle.quad(a, b, c, dt, dp, ddr, ddq)
    dt_g, dd_g = dt.copy(), np.zeros(N)
    dl, lp = np.zeros(1), np.zeros(1)
    rc = d.quad(P(np.array([a])), P(np.array([b])), P(np.array([c])), P(dt_g), P(dp), P(ddr), P(ddq), P(dd_g),
                P(dl), P(lp))
    assert rc == rc_o == 0
    assert abs(dl[0] - dl_o) < 1e-14 * abs(dl_o)
    assert _rel(dt_g, dt_o) < 1e-14 and _rel(dd_g, dd_o) < 1e-14
    assert d.quad(P(np.array([1.0])), P(np.array([0.0])), P(np.array([1.0])), P(dt_g), P(dp), P(ddr), P(ddq),
                  P(dd_g), P(dl), P(lp)) == 2
    vecs = [rng.normal(size=N) for _ in range(6)]
    for tol in ((1e-3, 1.0, 1.0), (1.0, 1e-1, 1.0), (1.0, 1.0, 1e-2), (10.0, 10.0, 10.0)):
        rc_o, cc_o = oracle.test_criteria(*vecs, 3.5, *tol)
        cc = np.zeros(1, dtype=np.int32)
        rc = d.test(*[P(v) for v in vecs], P(np.array([3.5])), P(cc), P(np.array([tol[0]])), P(np.array([tol[1]])),
                    P(np.array([tol[2]])))
        assert (rc, int(cc[0])) == (rc_o, cc_o)
    a1, b1 = rng.normal(size=N), rng.normal(size=N)
    assert abs(d.dot(P(a1), P(b1), N) - float(a1 @ b1)) < 1e-12 * np.abs(a1 * b1).sum()
