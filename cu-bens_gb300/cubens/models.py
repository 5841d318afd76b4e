"""Seeded generators for the CU-BENs benchmark models, written as model_def.txt text.

Every generator returns the text of a ``model_def.txt`` in the positional,
comma-separated layout that the reference reads:

* header and element counts          main.c:340-433
* incidences and constraints        model.c:95-264 (``struc``)
* joint coordinates                  main.c:1395-1397
* truss / shell properties           truss.c:66, shell.c:61
* joint loads                        model.c:1313-1335 (``load``)
* MSAL control block                 arc.c:48, main.c:2240-2245

The generators are deterministic. The only random input (the panel imperfection)
comes from ``numpy.random.default_rng(seed)``, and the seed is part of the
returned ``ModelSpec``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class MsalControls:
    """MSAL parameters in the order main.c:2240-2245 reads them."""

    joint: int            # joint of the initially prescribed displacement (1-based)
    direction: int        # 1..6
    dk: float             # initially prescribed displacement
    alpha: float = 1.0
    psi_thresh: float = 0.1
    iteopt: int = 6
    lpfmax: float = 1e9
    dkimax: float = 1e9
    itemax: int = 20
    submax: int = 10
    imagmax: int = 10
    negmax: int = 10
    toldisp: float = 1e-6
    tolforc: float = 1.0
    tolener: float = 1e-6

    def lines(self) -> list[str]:
        return [
            f"{self.joint},{self.direction},{self.dk!r}",
            f"{self.alpha!r}",
            f"{self.psi_thresh!r}",
            f"{self.iteopt}",
            f"{self.lpfmax!r},{self.dkimax!r}",
            f"{self.itemax},{self.submax},{self.imagmax},{self.negmax}",
            f"{self.toldisp!r},{self.tolforc!r},{self.tolener!r}",
        ]


@dataclass
class NewtonControls:
    """Static load-control parameters of the Newton-Raphson (alg 1) and
    modified Newton-Raphson (alg 2) loops, in the order main.c:1809-1812
    reads them."""

    alg: int = 1          # ALGFLAG: 1 Newton-Raphson, 2 modified Newton-Raphson
    lpfmax: float = 1.0
    lpf: float = 0.1
    dlpf: float = 0.1
    dlpfmax: float = 0.2
    dlpfmin: float = 0.0125
    itemax: int = 20
    submax: int = 8
    solmin: int = 2
    toldisp: float = 1e-8
    tolforc: float = 1.0
    tolener: float = 1e-8

    def lines(self) -> list[str]:
        return [
            f"{self.lpfmax!r},{self.lpf!r},{self.dlpf!r},{self.dlpfmax!r},{self.dlpfmin!r}",
            f"{self.itemax},{self.submax},{self.solmin}",
            f"{self.toldisp!r},{self.tolforc!r},{self.tolener!r}",
        ]


def _alg(controls) -> str:
    return str(controls.alg) if isinstance(controls, NewtonControls) else "3"


@dataclass
class ModelSpec:
    name: str
    text: str
    nj: int
    ne_tr: int = 0
    ne_fr: int = 0
    ne_sh: int = 0
    seed: int | None = None
    params: dict = field(default_factory=dict)


def _fmt(v: float) -> str:
    # repr() round-trips a double exactly through the reference's "%lf" fscanf.
    return repr(float(v))


def space_truss(bays: int = 10, bay: float = 3.0, depth: float = 1.5,
                emod: float = 200e9, area: float = 1.0e-3, load: float = -10e3,
                controls: MsalControls | None = None) -> ModelSpec:
    """Double-layer square space truss (10x10 bays of 3.0 m, depth 1.5 m).

    The top grid has (bays+1)^2 joints and the bottom grid bays^2 joints offset
    by half a bay. Top and bottom chords run along both axes; every bottom joint
    has four diagonals to the top corners of its bay. Perimeter top joints are
    pinned (translations fixed); every interior top joint carries ``load`` in
    direction 3. Truss joints expose DOF 1-3 only (model.c:267-285).
    """
    nb = bays
    nodes: list[tuple[float, float, float]] = []
    top: dict[tuple[int, int], int] = {}
    bot: dict[tuple[int, int], int] = {}
    for i in range(nb + 1):
        for j in range(nb + 1):
            nodes.append((bay * i, bay * j, depth))
            top[(i, j)] = len(nodes)
    for i in range(nb):
        for j in range(nb):
            nodes.append((bay * i + bay / 2, bay * j + bay / 2, 0.0))
            bot[(i, j)] = len(nodes)
    el: list[tuple[int, int]] = []
    for i in range(nb + 1):
        for j in range(nb):
            el.append((top[(i, j)], top[(i, j + 1)]))
            el.append((top[(j, i)], top[(j + 1, i)]))
    for i in range(nb):
        for j in range(nb - 1):
            el.append((bot[(i, j)], bot[(i, j + 1)]))
            el.append((bot[(j, i)], bot[(j + 1, i)]))
    for i in range(nb):
        for j in range(nb):
            for di in (0, 1):
                for dj in (0, 1):
                    el.append((bot[(i, j)], top[(i + di, j + dj)]))
    cons: list[str] = []
    loads: list[str] = []
    for (i, j), k in sorted(top.items(), key=lambda kv: kv[1]):
        if i in (0, nb) or j in (0, nb):
            cons += [f"{k},{d}" for d in (1, 2, 3)]
        else:
            loads.append(f"{k},3,{_fmt(load)}")
    centre = top[(nb // 2, nb // 2)]
    if controls is None:
        controls = MsalControls(joint=centre, direction=3, dk=-0.005,
                                toldisp=1e-10, tolforc=1.0, tolener=1e-10,
                                itemax=20)
    out = ["2", _alg(controls), "0", "1", str(len(nodes)), f"{len(el)},0,0,0,0"]
    out += [f"{a},{b}" for a, b in el]
    out += cons + ["0,0"]
    out += [f"{_fmt(x)},{_fmt(y)},{_fmt(z)}" for x, y, z in nodes]
    out += [f"{_fmt(emod)},{_fmt(area)},7850.0,1e30"] * len(el)
    out += loads + ["0,0,0"]
    out += controls.lines()
    return ModelSpec("space_truss", "\n".join(out) + "\n", nj=len(nodes),
                     ne_tr=len(el), params={"bays": nb, "centre": centre})


PANEL_R = 2540.0
PANEL_L = 508.0
PANEL_THETA = 0.2
PANEL_T = 12.7
PANEL_E = 3102.75
PANEL_NU = 0.3


def imperfection_amplitudes(seed: int, scale: float) -> np.ndarray:
    """Four sine-mode amplitudes ~ U(-scale, scale) * thickness, seeded."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-scale, scale, size=4) * PANEL_T


# (m, p) sine modes of the imperfection, axial x angular; the builder's choice.
IMPERFECTION_MODES = ((1, 1), (1, 2), (2, 1), (2, 2))


def cylindrical_panel(n: int = 64, seed: int | None = None, imperfection: float = 0.0,
                      load: float = -1.0, controls: MsalControls | None = None,
                      radius: float = PANEL_R, length: float = PANEL_L,
                      theta: float = PANEL_THETA, thick: float = PANEL_T,
                      emod: float = PANEL_E, nu: float = PANEL_NU, n_axial: int | None = None) -> ModelSpec:
    """Hinged cylindrical DKT shell panel on an n x n quad grid (2 n^2 triangles).

    With ``n_axial`` the grid has n_axial divisions along the axis and n
    around it (the band of the equations, set by the n + 1 joints of an
    axial station, stays that of the n x n panel).

    Joints are (x_i, R sin a_j, R cos a_j - R) with x_i = L i/n along the axis and
    a_j = -theta/2 + theta j/n; joint (i, j) is number i*(n+1)+j+1. Each quad
    (a,b,c,d) splits into (a,b,c) and (a,c,d). Both straight (axial) edges
    j=0 and j=n have translations 1-3 fixed; the curved edges are free. The
    centre joint carries ``load`` in direction 3. With ``seed`` given, a radial
    imperfection sum_k A_k sin(m_k pi x/L) sin(p_k pi (a+theta/2)/theta) is
    added, A_k ~ U(-imperfection, imperfection) * thickness.
    """
    amps = np.zeros(4)
    if seed is not None and imperfection > 0:
        amps = imperfection_amplitudes(seed, imperfection)
    na = n if n_axial is None else n_axial
    nodes = []
    for i in range(na + 1):
        x = length * i / na
        for j in range(n + 1):
            a = -theta / 2 + theta * j / n
            w = 0.0
            for (m, p), amp in zip(IMPERFECTION_MODES, amps):
                w += amp * math.sin(m * math.pi * x / length) * math.sin(p * math.pi * (a + theta / 2) / theta)
            r = radius + w
            nodes.append((x, r * math.sin(a), r * math.cos(a) - radius))

    def idx(i: int, j: int) -> int:
        return i * (n + 1) + j + 1

    tris = []
    for i in range(na):
        for j in range(n):
            a, b, c, d = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
            tris.append((a, b, c))
            tris.append((a, c, d))
    cons = []
    for i in range(na + 1):
        for j in (0, n):
            for dr in (1, 2, 3):
                cons.append(f"{idx(i, j)},{dr}")
    centre = idx(na // 2, n // 2)
    if controls is None:
        controls = MsalControls(joint=centre, direction=3, dk=-0.5)
    out = ["2", _alg(controls), "0", "1", str(len(nodes)), f"0,0,{len(tris)},0,0"]
    out += [f"{a},{b},{c}" for a, b, c in tris]
    out += cons + ["0,0"]
    out += [f"{_fmt(x)},{_fmt(y)},{_fmt(z)}" for x, y, z in nodes]
    out += [f"{_fmt(emod)},{_fmt(nu)},{_fmt(thick)},1.0,1e30"] * len(tris)
    out += [f"{centre},3,{_fmt(load)}", "0,0,0"]
    out += controls.lines()
    return ModelSpec(f"panel{n}", "\n".join(out) + "\n", nj=len(nodes), ne_sh=len(tris),
                     seed=seed, params={"n": n, "centre": centre,
                                        "imperfection_amplitudes": amps.tolist()})


def shell_panel_linear(n: int = 8, steps: int = 40, dt: float = 0.01, peak: float = -1.0,
                       numopt: int = 1, spectrds: float = 0.8, dens: float = 1.0) -> ModelSpec:
    """The hinged cylindrical panel of ``cylindrical_panel`` as a linear
    dynamic model (ANAFLAG 1, ALGFLAG 4, main.c:3143-3302): density ``dens``,
    a half-sine pulse of ``peak`` in direction 3 at the centre joint over the
    first quarter of the ``steps`` time steps of ``dt``, then free vibration;
    Newmark controls numopt and spectrds (main.c:3184) and lpfmax 1."""
    base = cylindrical_panel(n).text.splitlines()
    ne = 2 * n * n
    nj = (n + 1) * (n + 1)
    centre = n // 2 * (n + 1) + n // 2 + 1
    # the MSAL text: flags, incidences, constraints ... "0,0", coordinates,
    # properties, then the loads and controls, which are replaced
    i_cons_end = base.index("0,0")
    head = base[4:i_cons_end + 1]                     # NJ, counts, incidences, constraints, "0,0"
    coords = base[i_cons_end + 1:i_cons_end + 1 + nj]
    props = [f"{_fmt(PANEL_E)},{_fmt(PANEL_NU)},{_fmt(PANEL_T)},{_fmt(dens)},1e30"] * ne
    out = ["1", "4", "0,0", "0", "1"] + head + ["0,0"] + coords + props
    out.append(f"{steps},{_fmt(steps * dt)}")
    npulse = max(2, steps // 4)
    for k in range(steps + 1):
        v = peak * math.sin(math.pi * k / npulse) if k <= npulse else 0.0
        out.append(f"{centre},3,{_fmt(v)}")
    out += ["0,0,0", "0,0,0", "0,0,0,0,0", f"{numopt},{spectrds!r}", "1.0"]
    return ModelSpec(f"panel{n}_linear", "\n".join(out) + "\n", nj=nj, ne_sh=ne,
                     params={"n": n, "centre": centre, "steps": steps, "dt": dt})


def batch_sizes(count: int = 512, seed: int = 2024,
                choices: tuple[int, ...] = tuple(range(16, 97, 8))) -> list[int]:
    """Mesh sizes drawn uniformly from {16, 24, ..., 96}, seeded."""
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.choice(np.array(choices), size=count)]


@dataclass
class NewmarkControls:
    """Nonlinear Newmark parameters in the order main.c:3320-3326 reads them.

    numopt 0 with spectrds 1 gives alpha_m = alpha_f = 0, i.e. the average
    acceleration rule beta = 0.25, gamma = 0.5 (main.c:3329-3343)."""

    numopt: int = 0
    spectrds: float = 1.0
    lpfmax: float = 1.0
    lpf: float = 1.0
    dlpf: float = 1.0
    dlpfmax: float = 1.0
    dlpfmin: float = 1.0
    itemax: int = 20
    submax: int = 10
    solmin: int = 3
    toldisp: float = 1e-8
    tolforc: float = 1.0
    tolener: float = 1e-8

    def lines(self) -> list[str]:
        return [
            f"{self.numopt},{self.spectrds!r}",
            f"{self.lpfmax!r},{self.lpf!r},{self.dlpf!r},{self.dlpfmax!r},{self.dlpfmin!r}",
            f"{self.itemax},{self.submax},{self.solmin}",
            f"{self.toldisp!r},{self.tolforc!r},{self.tolener!r}",
        ]


FRAME_E = 200e9
FRAME_NU = 0.3
FRAME_RHO = 7850.0
COLUMN_A, COLUMN_I = 0.02, 2e-4
BEAM_A, BEAM_I = 0.012, 1e-4


def band_limited_noise(nt: int, dt: float, rms: float, seed: int,
                       band: tuple[float, float] = (0.5, 10.0)) -> np.ndarray:
    """Seeded Gaussian white noise, band-passed in the FFT domain to ``band`` Hz
    (bins outside the band zeroed) and scaled to the given RMS."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(nt)
    spec = np.fft.rfft(w)
    freq = np.fft.rfftfreq(nt, dt)
    spec[(freq < band[0]) | (freq > band[1])] = 0.0
    s = np.fft.irfft(spec, nt)
    r = math.sqrt(float(np.mean(s * s)))
    return s * (rms / r) if r > 0 else s


def frame_building(bays_x: int = 20, bays_y: int = 20, storeys: int = 30,
                   bay: float = 6.0, storey: float = 3.5, warping: str = "fixed",
                   steps: int = 2000, dt: float = 0.005, rms: float = 5e3, seed: int = 4,
                   loaded_face: bool = True, newmark: NewmarkControls | None = None,
                   msal: MsalControls | None = None, msal_load: float = 1e3, linear: bool = False,
                   initial: list | None = None) -> ModelSpec:
    """Rigid-jointed 3D frame building of co-rotational 14-DOF frame members.

    Joint (i, j, s) at (bay*i, bay*j, storey*s) is number
    s*(bx+1)*(by+1) + j*(bx+1) + i + 1. Columns join (i, j, s) to (i, j, s+1)
    and come first; then each floor s >= 1 has beams along x, then along y.
    The base joints (s = 0) are fixed. ``warping`` "fixed" writes "j,7,0" for
    every joint (6 DOF per joint); "member" writes "j,7,1" (one warping DOF per
    member end, model.c:941-961). Columns: A = 0.02, I = 2e-4; beams: A =
    0.012, I = 1e-4 (both bending axes); J = 2I, no warping constant; steel
    E = 200 GPa, nu = 0.3, rho = 7850. Aux points lie one unit along global x
    from a column's first joint and one unit up from a beam's first joint.

    Dynamic (default, ALGFLAG 5): every floor s >= 1 gets its own seeded
    band-limited (0.5-10 Hz) noise history scaled to ``rms`` N, applied in
    global x at each joint of the floor's x = 0 face (one history per floor,
    ``steps`` + 1 time points of ``dt``). With ``msal`` given the model is an
    MSAL model instead: ``msal_load`` in x at every joint of the roof's x = 0
    face is the reference load. With ``linear`` the dynamic model is the
    reference's linear one (ANAFLAG 1, ALGFLAG 4: one factorisation of the
    initial effective stiffness, main.c:3143-3302): its controls are
    ``newmark``'s numopt and spectrds and then lpfmax alone (main.c:3184,
    3192), and ``initial`` lists (joint, direction, d, v, a) initial
    conditions.
    """
    bx, by, ns = bays_x, bays_y, storeys
    nper = (bx + 1) * (by + 1)

    def jid(i: int, j: int, s: int) -> int:
        return s * nper + j * (bx + 1) + i + 1

    nodes = [(bay * i, bay * j, storey * s) for s in range(ns + 1) for j in range(by + 1)
             for i in range(bx + 1)]
    cols, beams = [], []
    for s in range(ns):
        for j in range(by + 1):
            for i in range(bx + 1):
                cols.append((jid(i, j, s), jid(i, j, s + 1)))
    for s in range(1, ns + 1):
        for j in range(by + 1):
            for i in range(bx):
                beams.append((jid(i, j, s), jid(i + 1, j, s)))
        for j in range(by):
            for i in range(bx + 1):
                beams.append((jid(i, j, s), jid(i, j + 1, s)))
    members = cols + beams
    gmod = FRAME_E / (2 * (1 + FRAME_NU))
    wflag = {"fixed": 0, "member": 1}[warping]
    cons = []
    for k in range(1, len(nodes) + 1):
        if k <= nper:
            cons += [f"{k},{d}" for d in range(1, 7)]
        cons.append(f"{k},7,{wflag}")
    props, aux = [], []
    for n, (a, b) in enumerate(members):
        col = n < len(cols)
        A, I = (COLUMN_A, COLUMN_I) if col else (BEAM_A, BEAM_I)
        props.append(f"{_fmt(FRAME_E)},{_fmt(gmod)},{_fmt(FRAME_RHO)},{_fmt(A)},{_fmt(I)},{_fmt(I)},"
                     f"{_fmt(2 * I)},0.0")
        x0 = nodes[a - 1]
        off = (1.0, 0.0, 0.0) if col else (0.0, 0.0, 1.0)
        aux.append(",".join(_fmt(x0[k] + off[k]) for k in range(3)))
    face = lambda s: [jid(0, j, s) for j in range(by + 1)]  # noqa: E731
    dynamic = msal is None
    if linear and not dynamic:
        raise ValueError("a linear (ALGFLAG 4) model is dynamic: give no msal controls")
    out = ["1" if linear else "2", ("4" if linear else "5") if dynamic else _alg(msal)]
    if dynamic:
        out.append("0,0")                     # CHKPT, RFLAG
    out += ["0", "1", str(len(nodes)), f"0,{len(members)},0,0,0"]
    out += [f"{a},{b}" for a, b in members]
    out += cons + ["0,0"]
    if dynamic:
        out.append("0,0")                     # no prescribed support motion
    out += [f"{_fmt(x)},{_fmt(y)},{_fmt(z)}" for x, y, z in nodes]
    out += props
    out.append("0,0,0,0,0,0,0")               # no member end offsets
    out += aux
    out += ["1e30,1.0,1.0"] * len(members)    # yield stress, plastic moduli (unused, ANAFLAG 2)
    out.append("0,0,0,0,0")                   # no member end releases
    params: dict = {"bays_x": bx, "bays_y": by, "storeys": ns, "columns": len(cols),
                    "beams": len(beams), "warping": warping}
    if dynamic:
        nt = steps + 1
        ttot = steps * dt
        out.append(f"{steps},{_fmt(ttot)}")
        for s in range(1, ns + 1):
            hist = band_limited_noise(nt, dt, rms, seed * 1000 + s)
            joints = face(s) if loaded_face else [jid(0, 0, s)]
            for jt in joints:
                out += [f"{jt},1,{_fmt(v)}" for v in hist]
        out += ["0,0,0", "0,0,0"]
        out += [f"{jt},{dr},{_fmt(d)},{_fmt(v)},{_fmt(a)}" for jt, dr, d, v, a in (initial or [])]
        out.append("0,0,0,0,0")
        nm = newmark or NewmarkControls()
        if linear:
            out += [f"{nm.numopt},{nm.spectrds!r}", f"{nm.lpfmax!r}"]
        else:
            out += nm.lines()
        params.update(steps=steps, dt=dt, rms=rms)
    else:
        out += [f"{jt},1,{_fmt(msal_load)}" for jt in face(ns)] + ["0,0,0"]
        out.append("0,0,0")                   # no distributed loads
        out += msal.lines()
    name = f"frame{bx}x{by}x{ns}" + ("" if dynamic else "_msal") + ("_linear" if linear else "")
    params["members"] = members               # 1-based joint pairs, in input order
    return ModelSpec(name, "\n".join(out) + "\n", nj=len(nodes), ne_fr=len(members),
                     seed=seed if dynamic else None, params=params)
