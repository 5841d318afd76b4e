"""ctypes binding of the CPU oracle (liboracle.so, built from cubens_oracle.c).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
_lib = None


def build(quiet: bool = True) -> Path:
    subprocess.run(["make", "-C", str(HERE), "liboracle.so"], check=True,
                   capture_output=quiet)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        dp = C.POINTER(C.c_double)
        lp = C.POINTER(C.c_long)
        ip = C.POINTER(C.c_int)
        L.orc_load.restype = P
        L.orc_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.orc_free.argtypes = [P]
        L.orc_sizes.argtypes = [P, lp]
        L.orc_topology.argtypes = [P, lp, dp]
        L.orc_msal.restype = C.c_int
        L.orc_msal.argtypes = [P, C.c_int, dp, ip, dp, dp, C.c_char_p, C.c_int]
        L.orc_msal_timed.restype = C.c_int
        L.orc_msal_timed.argtypes = [P, C.c_int, dp, ip, dp, dp, dp, C.c_char_p, C.c_int]
        L.orc_shell_forces.argtypes = [P, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_truss_forces.argtypes = [P, dp, dp, dp, dp, dp]
        L.orc_tangent.argtypes = [P, dp, dp, dp, dp, dp, dp, lp, dp]
        L.orc_skyline_solve.argtypes = [P, dp, dp, dp, ip, C.c_int]
        L.orc_shell_initial.argtypes = [P, dp, dp]
        L.orc_dyn_sizes.argtypes = [P, lp, dp]
        L.orc_linear_newmark.restype = C.c_int
        L.orc_linear_newmark.argtypes = [P, C.c_long, dp, dp, C.c_char_p, C.c_int]
        L.orc_newmark.restype = C.c_int
        L.orc_newmark.argtypes = [P, C.c_long, dp, ip, dp, dp, C.c_char_p, C.c_int]
        L.orc_frame_initial.argtypes = [P, dp, dp]
        L.orc_frame_forces.argtypes = [P, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_tangent_fr.argtypes = [P, dp, dp, dp, dp, lp, dp]
        L.orc_frame_mass.argtypes = [P, dp, dp]
        L.orc_frame_mcode.argtypes = [P, lp]
        L.orc_shell_geometry0.argtypes = [P, dp, dp]
        L.orc_quad.restype = C.c_int
        L.orc_quad.argtypes = [C.c_long, C.c_double, C.c_double, C.c_double, dp, dp, dp, dp, dp, dp, dp]
        L.orc_test.restype = C.c_int
        L.orc_test.argtypes = [C.c_long, dp, dp, dp, dp, dp, dp, C.c_double, ip, C.c_double, C.c_double,
                               C.c_double]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _l(a):
    return a.ctypes.data_as(C.POINTER(C.c_long))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class OracleModel:
    def __init__(self, text: str):
        err = C.create_string_buffer(256)
        self.h = lib().orc_load(text.encode(), err, 256)
        if not self.h:
            raise ValueError(err.value.decode())
        s = np.zeros(8, dtype=np.int64)
        lib().orc_sizes(self.h, _l(s))
        self.nj, self.ne_tr, self.ne_fr, self.ne_sh, self.neq, self.lss, self.dkdof, self.itemax = map(int, s)
        self.jcode = np.zeros(self.nj * 7, dtype=np.int64)
        self.q = np.zeros(self.neq)
        lib().orc_topology(self.h, _l(self.jcode), _d(self.q))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_free(self.h)
            self.h = None

    def msal(self, steps: int):
        lam = np.zeros(steps)
        its = np.zeros(steps, dtype=np.int32)
        d = np.zeros((steps, self.neq))
        res = np.zeros(steps)
        err = C.create_string_buffer(256)
        n = lib().orc_msal(self.h, steps, _d(lam), _i(its), _d(d), _d(res), err, 256)
        nconv = int(np.count_nonzero(its))
        return dict(rc=n, error=err.value.decode(), lam=lam[:nconv], its=its[:nconv],
                    d=d[:nconv], res=res[:nconv])

    def msal_timed(self, steps: int, keep_d: bool = False):
        """MSAL run with the wall time of every accepted step (seconds, monotonic)."""
        lam = np.zeros(steps)
        its = np.zeros(steps, dtype=np.int32)
        d = np.zeros((steps, self.neq)) if keep_d else None
        res = np.zeros(steps)
        ts = np.zeros(steps)
        err = C.create_string_buffer(256)
        n = lib().orc_msal_timed(self.h, steps, _d(lam), _i(its), _d(d) if keep_d else None, _d(res),
                                 _d(ts), err, 256)
        nconv = int(np.count_nonzero(its))
        return dict(rc=n, error=err.value.decode(), lam=lam[:nconv], its=its[:nconv], res=res[:nconv],
                    t=ts[:nconv], d=d[:nconv] if keep_d else None)

    def dyn_sizes(self):
        n = np.zeros(1, dtype=np.int64)
        dt = np.zeros(1)
        lib().orc_dyn_sizes(self.h, _l(n), _d(dt))
        return int(n[0]), float(dt[0])

    def newmark(self, steps: int, keep_d: bool = True):
        """Nonlinear Newmark run; per recorded time step: time, its, d, res."""
        t = np.zeros(steps)
        its = np.zeros(steps, dtype=np.int32)
        d = np.zeros((steps, self.neq)) if keep_d else None
        res = np.zeros(steps)
        err = C.create_string_buffer(256)
        n = lib().orc_newmark(self.h, steps, _d(t), _i(its), _d(d) if keep_d else None, _d(res), err, 256)
        k = max(n, 0)
        return dict(rc=n, error=err.value.decode(), time=t[:k], its=its[:k], res=res[:k],
                    d=d[:k] if keep_d else None)

    def linear_newmark(self, steps: int):
        """Linear Newmark run (ALGFLAG 4): per time step the time and d."""
        t = np.zeros(steps)
        d = np.zeros((steps, self.neq))
        err = C.create_string_buffer(256)
        n = lib().orc_linear_newmark(self.h, steps, _d(t), _d(d), err, 256)
        if n < 0:
            raise ValueError(err.value.decode())
        return dict(rc=n, time=t[:n], d=d[:n])

    def frame_initial(self):
        c = np.zeros(self.ne_fr * 9)
        L = np.zeros(self.ne_fr)
        lib().orc_frame_initial(self.h, _d(c), _d(L))
        return c, L

    def frame_mcode(self):
        mc = np.zeros(self.ne_fr * 14, dtype=np.int64)
        lib().orc_frame_mcode(self.h, _l(mc))
        return mc

    def frame_forces(self, x_temp, dd, c_ip, ef_ip, len_ip, lref):
        c_i = np.zeros(self.ne_fr * 9)
        len_i = np.zeros(self.ne_fr)
        ef_i = np.zeros(self.ne_fr * 14)
        f = np.zeros(self.neq)
        args = [np.ascontiguousarray(v, dtype=np.float64) for v in (x_temp, dd, c_ip, ef_ip, len_ip, lref)]
        lib().orc_frame_forces(self.h, *[_d(v) for v in args], _d(c_i), _d(len_i), _d(ef_i), _d(f))
        return c_i, len_i, ef_i, f

    def tangent_fr(self, c, ef, length, lref):
        maxa = np.zeros(self.neq + 1, dtype=np.int64)
        ss = np.zeros(self.lss)
        args = [np.ascontiguousarray(v, dtype=np.float64) for v in (c, ef, length, lref)]
        lib().orc_tangent_fr(self.h, *[_d(v) for v in args], _l(maxa), _d(ss))
        return maxa, ss

    def frame_mass(self, x):
        sm = np.zeros(self.neq)
        lib().orc_frame_mass(self.h, _d(np.ascontiguousarray(x, dtype=np.float64)), _d(sm))
        return sm

    def shell_geometry0(self):
        xl = np.zeros(self.ne_sh * 3)
        sl = np.zeros(self.ne_sh * 3)
        lib().orc_shell_geometry0(self.h, _d(xl), _d(sl))
        return xl, sl

    def shell_initial(self):
        c = np.zeros(self.ne_sh * 9)
        a = np.zeros(self.ne_sh)
        lib().orc_shell_initial(self.h, _d(c), _d(a))
        return c, a

    def shell_forces(self, x_temp, dd, c_ip, ef_ip):
        c_i = np.zeros(self.ne_sh * 9)
        a_i = np.zeros(self.ne_sh)
        ef_i = np.zeros(self.ne_sh * 18)
        f = np.zeros(self.neq)
        args = [np.ascontiguousarray(v, dtype=np.float64) for v in (x_temp, dd, c_ip, ef_ip)]
        lib().orc_shell_forces(self.h, *[_d(v) for v in args], _d(c_i), _d(a_i), _d(ef_i), _d(f))
        return c_i, a_i, ef_i, f

    def truss_forces(self, x_temp):
        L = np.zeros(self.ne_tr)
        dr = np.zeros(self.ne_tr * 3)
        ef = np.zeros(self.ne_tr * 2)
        f = np.zeros(self.neq)
        lib().orc_truss_forces(self.h, _d(np.ascontiguousarray(x_temp, dtype=np.float64)),
                               _d(L), _d(dr), _d(ef), _d(f))
        return L, dr, ef, f

    def tangent(self, x, c_sh, a_sh, len_tr, dir_tr, ef_tr):
        maxa = np.zeros(self.neq + 1, dtype=np.int64)
        ss = np.zeros(self.lss)
        args = [np.ascontiguousarray(v, dtype=np.float64) for v in (x, c_sh, a_sh, len_tr, dir_tr, ef_tr)]
        lib().orc_tangent(self.h, *[_d(v) for v in args], _l(maxa), _d(ss))
        return maxa, ss

    def skyline_solve(self, ss, rhs, fact=0):
        ss = np.array(ss, dtype=np.float64)
        v = np.array(rhs, dtype=np.float64)
        ssd = np.zeros(self.neq)
        det = np.zeros(1, dtype=np.int32)
        lib().orc_skyline_solve(self.h, _d(ss), _d(v), _d(ssd), _i(det), fact)
        return v, ssd, int(det[0]), ss


def quad(a, b, c, dt, dp, ddr, ddq):
    """arc.c quad on copies: returns (status, dt, dd, dlpf, lpft increment)."""
    dt = np.array(dt, dtype=np.float64)
    dd = np.zeros_like(dt)
    dl = np.zeros(1)
    lp = np.zeros(1)
    rc = lib().orc_quad(len(dt), a, b, c, _d(dt), _d(np.ascontiguousarray(dp, dtype=np.float64)),
                        _d(np.ascontiguousarray(ddr, dtype=np.float64)),
                        _d(np.ascontiguousarray(ddq, dtype=np.float64)), _d(dd), _d(dl), _d(lp))
    return rc, dt, dd, float(dl[0]), float(lp[0])


def test_criteria(d_temp, dd, f_temp, fp, qtot, f_ip, intener1, toldisp, tolforc, tolener):
    """misc.c test: returns (status, convchk)."""
    cc = np.zeros(1, dtype=np.int32)
    args = [np.ascontiguousarray(v, dtype=np.float64) for v in (d_temp, dd, f_temp, fp, qtot, f_ip)]
    rc = lib().orc_test(len(args[0]), *[_d(v) for v in args], intener1, _i(cc), toldisp, tolforc, tolener)
    return rc, int(cc[0])


def skyline_to_dense(maxa, ss, neq):
    """Expand the 1-based skyline (upper triangle by columns) to a dense symmetric matrix."""
    K = np.zeros((neq, neq))
    for j in range(1, neq + 1):
        h = maxa[j] - maxa[j - 1] - 1
        for off in range(h + 1):
            i = j - off
            K[i - 1, j - 1] = K[j - 1, i - 1] = ss[maxa[j - 1] - 1 + off]
    return K
