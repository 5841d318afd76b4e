"""Generate the golden vectors that pin the oracle and the GPU path.

Every number written here comes from the reference's own compiled code, built
unmodified from its sources by ``make -C oracle ref``:

* whole-run fixtures: the reference driver (oracle/_ref/cuben_ref, main.c's
  MSAL loop) run on seeded models, with every converged step's lambda,
  iteration count and FP64 displacement vector dumped by the output() shim;
  The Newmark fixtures run main.c's ALGFLAG 5 loop the same way and record,
  per time step, the time (in the "lam" slot), iteration count and d; the
  Newton-Raphson fixtures (ALGFLAG 1 and 2) record every converged load
  increment's lpf, iteration count and d;
* element fixtures: the reference's prop_sh/prop_tr/prop_fr, updatc,
  forces_sh, forces_tr, forces_fr, stiff_sh, stiff_tr, stiff_fr, mass_fr,
  skyfact and skysolve called through oracle/_ref/libcuben_ref_elem.so on
  seeded random states.

Run in a tree that has the reference (it is not needed to *use* the fixtures):

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "cu-bens_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

from cubens import models  # noqa: E402
import oracle  # noqa: E402
import refrun  # noqa: E402

OUT = Path(__file__).resolve().parent
ELEM_LIB = ROOT / "oracle" / "_ref" / "libcuben_ref_elem.so"


def truss_controls() -> models.MsalControls:
    # psi_thresh > 1 keeps the load term out of the arc length (the 10 kN
    # reference load would otherwise dominate it); 1e-10 displacement and
    # energy tolerances, force criterion disabled (tolerance >= 1).
    return models.MsalControls(joint=61, direction=3, dk=-0.005, psi_thresh=1.1,
                               toldisp=1e-10, tolforc=1.0, tolener=1e-10, itemax=20)


def panel_controls(n: int, toldisp: float = 1e-5) -> models.MsalControls:
    # Displacement criterion only: the reference's DKT update leaves a drift
    # floor (drilling rotations carry stiffness but no internal force) that the
    # energy and force criteria cannot pass at useful arc lengths.
    centre = n // 2 * (n + 1) + n // 2 + 1
    return models.MsalControls(joint=centre, direction=3, dk=-0.2, toldisp=toldisp,
                               tolforc=1.0, tolener=1.0, itemax=100)


def frame_msal_controls(nj: int) -> models.MsalControls:
    # lateral roof displacement control at the last joint; the path passes a
    # limit point within 40 steps
    return models.MsalControls(joint=nj, direction=1, dk=0.2, toldisp=1e-8, tolforc=1.0,
                               tolener=1e-8, itemax=20)


def frame_msal_model(warping: str = "member") -> models.ModelSpec:
    nj = models.frame_building(2, 2, 3, msal=models.MsalControls(1, 1, 0.1)).nj
    return models.frame_building(2, 2, 3, warping=warping, msal=frame_msal_controls(nj), msal_load=1.0)


def frame_newmark_model(warping: str = "fixed", steps: int = 40) -> models.ModelSpec:
    return models.frame_building(2, 2, 3, warping=warping, steps=steps, dt=0.005, seed=4)


def whole_runs():
    cases = {
        "frame_msal": (frame_msal_model("member"), 40),
        "frame_newmark_fixed": (frame_newmark_model("fixed"), 41),
        "frame_newmark_member": (frame_newmark_model("member", 30), 31),
        "truss_c1": (models.space_truss(controls=truss_controls()), 50),
        "panel8": (models.cylindrical_panel(8, controls=panel_controls(8)), 12),
        "panel16_imp": (models.cylindrical_panel(16, seed=7, imperfection=0.1,
                                                 controls=panel_controls(16, 1e-4)), 8),
    }
    for name, (m, steps) in cases.items():
        r = refrun.run(m.text, steps, timeout=1200)
        assert r["returncode"] == 0, r["results1"][-400:]
        np.savez_compressed(OUT / f"run_{name}.npz", model_def=np.array(m.text),
                            steps=r["steps"], iterations=r["iterations"], lam=r["lam"],
                            d=r["d"], neq=r["neq"])
        print(name, "neq", r["neq"], "steps", len(r["lam"]), "its", r["iterations"].tolist())


def newton_cases():
    """Static Newton-Raphson (alg 1) and modified Newton-Raphson (alg 2) runs:
    load control below the panel's limit point, and the truss."""
    N = models.NewtonControls
    return {
        "truss_nr": (models.space_truss(controls=N(alg=1, lpfmax=1.5, lpf=0.1, dlpf=0.1, dlpfmax=0.4,
                                                   toldisp=1e-10, tolener=1e-10)), 20),
        "truss_mnr": (models.space_truss(controls=N(alg=2, lpfmax=1.5, lpf=0.1, dlpf=0.1, dlpfmax=0.4, itemax=60,
                                                    toldisp=1e-10, tolener=1e-10)), 20),
        "panel8_nr": (models.cylindrical_panel(8, controls=N(alg=1, lpfmax=85.0, lpf=10.0, dlpf=10.0, dlpfmax=20.0,
                                                             dlpfmin=0.625, toldisp=1e-5, tolener=1.0)), 20),
        "panel8_mnr": (models.cylindrical_panel(8, controls=N(alg=2, lpfmax=60.0, lpf=10.0, dlpf=10.0,
                                                              dlpfmax=20.0, dlpfmin=0.625, itemax=100,
                                                              toldisp=1e-5, tolener=1.0)), 20),
    }
    # Frames are left out: on the frame buildings the reference's static loop
    # reports a non-positive pivot, solves on the partly factored matrix
    # (solve ignores skyfact's error) and returns NaN displacements.


def newton_runs():
    for name, (m, steps) in newton_cases().items():
        r = refrun.run(m.text, steps, timeout=600)
        assert r["returncode"] == 0 and len(r["lam"]) > 0, r["results1"][-400:]
        np.savez_compressed(OUT / f"run_{name}.npz", model_def=np.array(m.text),
                            steps=r["steps"], iterations=r["iterations"], lam=r["lam"],
                            d=r["d"], neq=r["neq"], results_tail=np.array(r["results1"][-200:]))
        print(name, "neq", r["neq"], "incs", len(r["lam"]), "its", r["iterations"].tolist())


def results_cases():
    return {
        "truss_msal": (models.space_truss(controls=truss_controls()), 3),
        "panel8_msal": (models.cylindrical_panel(8, controls=panel_controls(8)), 4),
        "frame_newmark": (frame_newmark_model("fixed", 6), 5),
        "truss_nr": (newton_cases()["truss_nr"][0], 20),
    }


def results_fixtures():
    """The reference's own results2..5.txt (output(), misc.c:345-451) for
    short runs of each driver and element type."""
    texts, files = [], []
    names = list(results_cases())
    for name in names:
        m, steps = results_cases()[name]
        r = refrun.run(m.text, steps, timeout=600)
        assert r["returncode"] == 0, r["results1"][-400:]
        texts.append(m.text)
        files.append([r["results"].get(k, "") for k in range(2, 6)])
        print("results", name, [len(f) for f in files[-1]])
    np.savez_compressed(OUT / "results_files.npz", names=np.array(names), model_def=np.array(texts),
                        files=np.array(files), steps=np.array([results_cases()[n][1] for n in names]))


def linear_cases():
    """Linear Newmark frames (ANAFLAG 1, ALGFLAG 4) with initial conditions:
    numopt 1 (HHT-type dissipation, so the K u_m term of the effective load
    is active), warping fixed and one warping DOF per member end."""
    nm = models.NewmarkControls(numopt=1, spectrds=0.8)
    init = [(20, 1, 0.001, 0.01, 0.0), (30, 2, 0.0, -0.02, 0.5)]
    return {w: models.frame_building(2, 2, 3, warping=w, steps=40, dt=0.005, seed=3, linear=True, newmark=nm,
                                     initial=init)
            for w in ("fixed", "member")}


def linear_runs():
    """The reference's own linear Newmark runs: per time step the time and d
    (output() records; the reference's closing record, lpfmax with zero d, is
    dropped). Frames (warping fixed and per member) and the DKT panel with
    its lumped shell mass (mass_sh)."""
    cases = {f"frame_linear_{w}": m for w, m in linear_cases().items()}
    cases["panel8_linear"] = models.shell_panel_linear(8, steps=40, dt=0.01)
    for name, m in cases.items():
        r = refrun.run(m.text, 1000, timeout=600)
        assert r["returncode"] == 0, r["results1"][-400:]
        n = len(r["lam"]) - 1
        np.savez_compressed(OUT / f"run_{name}.npz", model_def=np.array(m.text), time=r["lam"][:n],
                            d=r["d"][:n], neq=r["neq"], results_tail=np.array(r["results1"][-200:]))
        print("linear", name, "neq", r["neq"], "steps", n)


def results1_cases():
    """Models whose whole results1.txt (the input echo and the run's
    messages) is pinned: the results2-5 cases, the frame with one warping DOF
    per member end (MSAL and Newmark), and an arc-length run whose first
    increment does not converge."""
    c = dict(results_cases())
    c["frame_msal_member"] = (frame_msal_model("member"), 3)
    c["frame_newmark_member"] = (frame_newmark_model("member", 6), 5)
    bad = models.MsalControls(joint=41, direction=3, dk=-50.0, toldisp=1e-5, tolforc=1.0, tolener=1.0, itemax=5)
    c["panel8_too_large"] = (models.cylindrical_panel(8, controls=bad), 2)
    return c


def results1_fixtures():
    """The reference's own results1.txt for the results1 cases."""
    texts, files, names = [], [], list(results1_cases())
    for name in names:
        m, steps = results1_cases()[name]
        r = refrun.run(m.text, steps, timeout=600)
        texts.append(m.text)
        files.append(r["results1"])
        print("results1", name, r["returncode"], len(r["results1"]), repr(r["results1"][-80:]))
    np.savez_compressed(OUT / "results1_files.npz", names=np.array(names), model_def=np.array(texts),
                        results1=np.array(files), steps=np.array([results1_cases()[n][1] for n in names]))


class RefElem:
    """The reference's element routines, called through the harness library."""

    def __init__(self):
        self.L = C.CDLL(str(ELEM_LIB))

    def sizes(self, nj, ne_tr, ne_sh, neq):
        self.L.href_set_sizes(C.c_long(nj), C.c_long(ne_tr), C.c_long(0), C.c_long(ne_sh),
                              C.c_long(neq), C.c_int(2), C.c_int(3))

    def read_props(self, text: str):
        f = tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False)
        f.write(text)
        f.close()
        assert self.L.href_open_input(f.name.encode()) == 0


def p(a):
    return a.ctypes.data_as(C.c_void_p)


def shell_element_fixture(n: int = 8, seed: int = 11):
    m = models.cylindrical_panel(n, controls=panel_controls(n))
    o = oracle.OracleModel(m.text)
    rng = np.random.default_rng(seed)
    R = RefElem()
    E, NJ, NEQ = o.ne_sh, o.nj, o.neq
    R.sizes(NJ, 0, E, NEQ)
    lines = m.text.splitlines()
    # the model_def lines after the coordinates are the E property lines
    head = 6 + E
    ncons = lines[head:].index("0,0") + 1
    x0 = np.array([[float(v) for v in ln.split(",")] for ln in lines[head + ncons:head + ncons + NJ]])
    props = "\n".join(lines[head + ncons + NJ:head + ncons + NJ + E]) + "\n"
    R.read_props(props)
    x = np.ascontiguousarray(x0.reshape(-1))
    emod, nu, thick, dens, yld = (np.zeros(E) for _ in range(5))
    xlocal, slength = np.zeros(3 * E), np.zeros(3 * E)
    farea = np.zeros(E)
    c1, c2, c3 = np.zeros(3 * E), np.zeros(3 * E), np.zeros(3 * E)
    minc = np.array([[int(v) for v in ln.split(",")] for ln in lines[6:6 + E]], dtype=np.int64).reshape(-1)
    R.L.prop_sh(p(x), p(emod), p(nu), p(xlocal), p(thick), p(dens), p(farea), p(slength), p(yld),
                p(c1), p(c2), p(c3), p(minc))
    jcode = o.jcode.copy()
    mcode = np.zeros(18 * E, dtype=np.int64)
    for s in range(E):
        for a in range(3):
            for d in range(6):
                mcode[s * 18 + a * 6 + d] = jcode[(minc[s * 3 + a] - 1) * 7 + d]
    zeros = np.zeros(max(1, 18 * E))
    x_ip = np.zeros(3 * NJ)
    defl = np.zeros(1)
    dfarea = np.zeros(E)
    dslen = np.zeros(3 * E)
    osflag = np.zeros(1, dtype=np.int32)

    def updatc(xt, dd, cc1, cc2, cc3, da, ds):
        R.L.updatc(p(xt), p(x_ip), p(zeros), p(dd), p(defl), p(da), p(ds), p(zeros), p(osflag),
                   p(zeros), p(cc1), p(cc2), p(cc3), p(minc), p(jcode))

    # state A: a prior displacement; its geometry gives c_ip
    x_temp = x.copy()
    dd1 = rng.normal(scale=0.5, size=NEQ)
    c1_ip, c2_ip, c3_ip = c1.copy(), c2.copy(), c3.copy()
    updatc(x_temp, dd1, c1_ip, c2_ip, c3_ip, dfarea, dslen)
    x_before = x_temp.copy()
    # state B: the increment whose forces we evaluate
    dd2 = rng.normal(scale=0.05, size=NEQ)
    c1_i, c2_i, c3_i = c1.copy(), c2.copy(), c3.copy()
    dfarea_i, dslen_i = np.zeros(E), np.zeros(3 * E)
    updatc(x_temp, dd2, c1_i, c2_i, c3_i, dfarea_i, dslen_i)
    ef_ip = rng.normal(scale=10.0, size=18 * E)
    ef_ip_in = ef_ip.copy()
    ef_i = np.zeros(18 * E)
    f = np.zeros(NEQ)
    d_temp = np.zeros(NEQ)
    chi = np.zeros(3 * E)
    efN = np.zeros(9 * E)
    efM = np.zeros(9 * E)
    dfarea_ip = dfarea.copy()
    dslen_ip = dslen.copy()
    R.L.forces_sh(p(f), p(ef_ip), p(ef_i), p(efN), p(efM), p(dd2), p(d_temp), p(chi), p(x_temp),
                  p(x_ip), p(emod), p(nu), p(xlocal), p(thick), p(farea), p(dfarea_ip), p(slength),
                  p(dslen_ip), p(yld), p(c1_ip), p(c2_ip), p(c3_ip), p(c1_i), p(c2_i), p(c3_i),
                  p(minc), p(mcode), p(jcode))
    # tangent at state B as the converged configuration, then LDL^T
    maxa = np.zeros(NEQ + 1, dtype=np.int64)
    lss = o.lss
    ss = np.zeros(lss)
    maxa_o, _ = o.tangent(x_temp, np.zeros(9 * E), np.ones(E), np.zeros(0), np.zeros(0), np.zeros(0))
    maxa[:] = maxa_o
    ef_conv = ef_i.copy()
    R.L.stiff_sh(p(ss), p(emod), p(nu), p(x_temp), p(xlocal), p(thick), p(farea), p(dfarea_i),
                 p(slength), p(dslen_i), p(yld), p(c1_i), p(c2_i), p(c3_i), p(ef_conv), p(d_temp),
                 p(chi), p(efN), p(efM), p(maxa), p(minc), p(mcode))
    ss_tangent = ss.copy()
    rhs = o.q.copy()
    ssd = np.zeros(NEQ)
    det = np.zeros(1, dtype=np.int32)
    R.L.skyfact(p(maxa), p(ss), p(ssd), p(rhs), C.c_int(0), p(det))
    R.L.skysolve(p(maxa), p(ss), p(ssd), p(rhs), C.c_int(0), p(det))

    def triads(a1, a2, a3):
        return np.stack([a1.reshape(E, 3), a2.reshape(E, 3), a3.reshape(E, 3)], axis=1).reshape(-1)

    np.savez_compressed(OUT / "elem_shell_panel8.npz", model_def=np.array(m.text),
                        x_before=x_before, dd=dd2, c_ip=triads(c1_ip, c2_ip, c3_ip),
                        ef_ip=ef_ip_in, x_after=x_temp, c_i=triads(c1_i, c2_i, c3_i),
                        area_i=dfarea_i, ef_i=ef_i, f=f, maxa=maxa, ss=ss_tangent,
                        ldlt_solution=rhs, ssd=ssd, det=det[0])
    print("shell element fixture: E", E, "NEQ", NEQ, "lss", lss, "det", det[0])


def truss_element_fixture(seed: int = 5):
    m = models.space_truss(controls=truss_controls())
    o = oracle.OracleModel(m.text)
    rng = np.random.default_rng(seed)
    R = RefElem()
    T, NJ, NEQ = o.ne_tr, o.nj, o.neq
    R.sizes(NJ, T, 0, NEQ)
    lines = m.text.splitlines()
    head = 6 + T
    ncons = lines[head:].index("0,0") + 1
    x0 = np.array([[float(v) for v in ln.split(",")] for ln in lines[head + ncons:head + ncons + NJ]])
    R.read_props("\n".join(lines[head + ncons + NJ:head + ncons + NJ + T]) + "\n")
    x = np.ascontiguousarray(x0.reshape(-1))
    emod, area, dens, llen, yld = (np.zeros(T) for _ in range(5))
    c1, c2, c3 = np.zeros(T), np.zeros(T), np.zeros(T)
    minc = np.array([[int(v) for v in ln.split(",")] for ln in lines[6:6 + T]], dtype=np.int64).reshape(-1)
    R.L.prop_tr(p(x), p(emod), p(area), p(dens), p(llen), p(yld), p(c1), p(c2), p(c3), p(minc))
    jcode = o.jcode.copy()
    mcode = np.zeros(6 * T, dtype=np.int64)
    for e in range(T):
        for a in range(2):
            for d in range(3):
                mcode[e * 6 + a * 3 + d] = jcode[(minc[e * 2 + a] - 1) * 7 + d]
    dd = rng.normal(scale=0.01, size=NEQ)
    x_temp = x.copy()
    x_ip = np.zeros(3 * NJ)
    defl_i = np.zeros(T)
    c1_i, c2_i, c3_i = c1.copy(), c2.copy(), c3.copy()
    z = np.zeros(18)
    osflag = np.zeros(1, dtype=np.int32)
    R.L.updatc(p(x_temp), p(x_ip), p(z), p(dd), p(defl_i), p(z), p(z), p(z), p(osflag), p(z),
               p(c1_i), p(c2_i), p(c3_i), p(minc), p(jcode))
    ef_i = np.zeros(2 * T)
    f = np.zeros(NEQ)
    R.L.forces_tr(p(f), p(ef_i), p(dd), p(emod), p(area), p(llen), p(defl_i), p(yld), p(c1_i),
                  p(c2_i), p(c3_i), p(mcode))
    maxa = np.zeros(NEQ + 1, dtype=np.int64)
    maxa[:], _ = o.tangent(x_temp, np.zeros(0), np.zeros(0), np.ones(T), np.zeros(3 * T), np.zeros(2 * T))
    ss = np.zeros(o.lss)
    R.L.stiff_tr(p(ss), p(emod), p(area), p(llen), p(defl_i), p(yld), p(c1_i), p(c2_i), p(c3_i),
                 p(ef_i), p(maxa), p(mcode))
    np.savez_compressed(OUT / "elem_truss_c1.npz", model_def=np.array(m.text), x_after=x_temp,
                        dd=dd, length_i=defl_i, dir_i=np.stack([c1_i, c2_i, c3_i], axis=1).reshape(-1),
                        ef_i=ef_i, f=f, maxa=maxa, ss=ss)
    print("truss element fixture: T", T, "NEQ", NEQ)


def frame_element_fixture(seed: int = 9):
    m = frame_msal_model("member")
    o = oracle.OracleModel(m.text)
    rng = np.random.default_rng(seed)
    R = RefElem()
    F, NJ, NEQ = o.ne_fr, o.nj, o.neq
    R.L.href_set_sizes(C.c_long(NJ), C.c_long(0), C.c_long(F), C.c_long(0), C.c_long(NEQ),
                       C.c_int(2), C.c_int(3))
    lines = m.text.splitlines()
    head = 6 + F
    ncons = lines[head:].index("0,0") + 1
    x0 = np.array([[float(v) for v in ln.split(",")] for ln in lines[head + ncons:head + ncons + NJ]])
    # property lines, offsets terminator, aux points, yield lines, releases terminator
    k0 = head + ncons + NJ
    R.read_props("\n".join(lines[k0:k0 + 3 * F + 2]) + "\n")
    x = np.ascontiguousarray(x0.reshape(-1))
    emod, gmod, dens, carea, llen = (np.zeros(F) for _ in range(5))
    istr, iweak, ipol, iwarp, yld, zs, zw = (np.zeros(F) for _ in range(7))
    xfr, offset, auxpt = np.zeros(6 * F), np.zeros(6 * F), np.zeros(3 * F)
    osflag = np.zeros(F, dtype=np.int32)
    mendrel = np.zeros(5 * F, dtype=np.int32)
    c1, c2, c3 = np.zeros(3 * F), np.zeros(3 * F), np.zeros(3 * F)
    minc = np.array([[int(v) for v in ln.split(",")] for ln in lines[6:6 + F]], dtype=np.int64).reshape(-1)
    R.L.prop_fr(p(x), p(xfr), p(emod), p(gmod), p(dens), p(offset), p(osflag), p(auxpt), p(carea),
                p(llen), p(istr), p(iweak), p(ipol), p(iwarp), p(yld), p(zs), p(zw), p(c1), p(c2),
                p(c3), p(mendrel), p(minc))
    jcode = o.jcode.copy()
    mcode = o.frame_mcode()
    x_ip = np.zeros(3 * NJ)
    z = np.zeros(max(1, 3 * F))

    def updatc(xt, dd, cc1, cc2, cc3, dl):
        xfr_t = xfr.copy()
        R.L.updatc(p(xt), p(x_ip), p(xfr_t), p(dd), p(dl), p(z), p(z), p(offset), p(osflag),
                   p(auxpt), p(cc1), p(cc2), p(cc3), p(minc), p(jcode))

    x_temp = x.copy()
    dd1 = rng.normal(scale=0.05, size=NEQ)
    c1_ip, c2_ip, c3_ip = c1.copy(), c2.copy(), c3.copy()
    len_ip = np.zeros(F)
    updatc(x_temp, dd1, c1_ip, c2_ip, c3_ip, len_ip)
    x_before = x_temp.copy()
    dd2 = rng.normal(scale=0.01, size=NEQ)
    c1_i, c2_i, c3_i = c1.copy(), c2.copy(), c3.copy()
    len_i = np.zeros(F)
    updatc(x_temp, dd2, c1_i, c2_i, c3_i, len_i)
    ef_ip = rng.normal(scale=1e4, size=14 * F)
    ef_ip_in = ef_ip.copy()
    ef_i = np.zeros(14 * F)
    efFE = np.zeros(14 * F)
    efFE_ip, efFE_i = np.zeros(14 * F), np.zeros(14 * F)
    yldflag = np.zeros(2 * F, dtype=np.int32)
    f = np.zeros(NEQ)
    dlpf = np.zeros(1)
    itecnt = np.zeros(1, dtype=np.int32)
    rc = R.L.forces_fr(p(f), p(ef_ip), p(ef_i), p(efFE), p(efFE_ip), p(efFE_i), p(yldflag), p(dd2),
                       p(emod), p(gmod), p(carea), p(offset), p(osflag), p(llen), p(len_ip), p(istr),
                       p(iweak), p(ipol), p(iwarp), p(yld), p(zs), p(zw), p(c1_ip), p(c2_ip), p(c3_ip),
                       p(c1_i), p(c2_i), p(c3_i), p(mendrel), p(mcode), p(dlpf), p(itecnt))
    assert rc == 0
    maxa = o.tangent_fr(np.zeros(9 * F), np.zeros(14 * F), np.ones(F), np.ones(F))[0]
    ss = np.zeros(o.lss)
    R.L.stiff_fr(p(ss), p(emod), p(gmod), p(carea), p(offset), p(osflag), p(llen), p(len_i), p(istr),
                 p(iweak), p(ipol), p(iwarp), p(yldflag), p(yld), p(zs), p(zw), p(c1_i), p(c2_i),
                 p(c3_i), p(ef_i), p(efFE_i), p(mendrel), p(maxa), p(mcode))
    sm = np.zeros(NEQ)
    lmass = llen.copy()
    xfr_m = xfr.copy()
    jac = np.zeros(1)
    R.L.mass_fr(p(sm), p(carea), p(lmass), p(istr), p(iweak), p(ipol), p(iwarp), p(dens), p(osflag),
                p(offset), p(x_temp), p(xfr_m), p(minc), p(mcode), p(jac))

    def triads(a1, a2, a3):
        return np.stack([a1.reshape(F, 3), a2.reshape(F, 3), a3.reshape(F, 3)], axis=1).reshape(-1)

    np.savez_compressed(OUT / "elem_frame_2x2x3.npz", model_def=np.array(m.text), x_before=x_before,
                        dd=dd2, c_ip=triads(c1_ip, c2_ip, c3_ip), ef_ip=ef_ip_in, len_ip=len_ip,
                        lref=llen, x_after=x_temp, c_i=triads(c1_i, c2_i, c3_i), len_i=len_i,
                        ef_i=ef_i, f=f, maxa=maxa, ss=ss, sm=sm, mass_len=lmass)
    print("frame element fixture: F", F, "NEQ", NEQ, "lss", o.lss)


if __name__ == "__main__":
    oracle.build()
    frame_element_fixture()
    shell_element_fixture()
    truss_element_fixture()
    whole_runs()
    newton_runs()
    results_fixtures()
    results1_fixtures()
    linear_runs()
