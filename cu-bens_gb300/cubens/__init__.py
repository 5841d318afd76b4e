"""cubens_gb300: GB300 (sm_103a) hot path of CU-BENs behind a C ABI.

This package is the Python host mirror of the C ABI in include/cubens_gb300.h.
It loads the in-tree CUDA library (cu-bens_gb300/lib/libcubens_gb300.so,
built by ``cubens.build.build()``) through ctypes. There is no CPU fallback:
if the library is missing or no GPU is present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build as _build
from . import models  # noqa: F401  (re-exported generators)

LIB_PATH = _build.LIB

CB_OK = 0
STATUS = {0: "ok", 1: "bad argument", 2: "parse error", 3: "CUDA error", 4: "unsupported",
          5: "numeric failure", 6: "diverged", 7: "bad call order", 8: "timeout", 9: "limit"}

FP64 = 0
MIXED = 1
FP32X2 = 2

K_SOLVE, K_SHELL_FORCE, K_FACTOR, K_BAND_LDLT, K_SOLVE_BLOCKS, K_FRAME_FORCE, K_SPMV = range(7)

SOLVER_BAND, SOLVER_FGMRES = 0, 1
PRECOND_BLOCK_JACOBI, PRECOND_LEARNED = 0, 1


class CubensError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("use_graphs", C.c_int),
                ("solver", C.c_int), ("krylov_restart", C.c_int), ("krylov_maxit", C.c_int),
                ("precond", C.c_int), ("factor_kernel", C.c_int), ("band_solve", C.c_int)]


class Info(C.Structure):
    _fields_ = [("nj", C.c_long), ("ne_tr", C.c_long), ("ne_fr", C.c_long), ("ne_sh", C.c_long),
                ("neq", C.c_long), ("lss", C.c_long), ("bandwidth", C.c_long), ("block", C.c_long),
                ("nblocks", C.c_long), ("dkdof", C.c_long), ("device_bytes", C.c_size_t),
                ("h2d_bytes", C.c_size_t), ("algflag", C.c_int), ("nsteps", C.c_long), ("dt", C.c_double),
                ("solver", C.c_int), ("nnz", C.c_long), ("node_blocks", C.c_long), ("factor_cluster", C.c_int)]


class Step(C.Structure):
    _fields_ = [("lam", C.c_double), ("iterations", C.c_int), ("attempts", C.c_int),
                ("residual", C.c_double), ("dk", C.c_double), ("done", C.c_int)]


class Timers(C.Structure):
    _fields_ = [("ms_tangent", C.c_double), ("ms_factor", C.c_double), ("ms_solve", C.c_double),
                ("ms_force", C.c_double), ("ms_vector", C.c_double), ("launches", C.c_long),
                ("solves", C.c_long), ("factorizations", C.c_long), ("force_evals", C.c_long),
                ("ms_train", C.c_double)]


class KrylovStats(C.Structure):
    _fields_ = [("solves", C.c_long), ("iterations", C.c_long), ("unconverged", C.c_long),
                ("last_iterations", C.c_int), ("last_residual", C.c_double), ("learned_solves", C.c_long),
                ("fallbacks", C.c_long), ("train_steps", C.c_long), ("train_loss", C.c_double),
                ("inner_iterations", C.c_long)]


_lib = None


def load(path: Path | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with cubens.build.build() (nvcc, sm_103a)")
    L = C.CDLL(str(p))
    dp = C.POINTER(C.c_double)
    lp = C.POINTER(C.c_long)
    ip = C.POINTER(C.c_int)
    vp = C.c_void_p
    L.cb_default_options.argtypes = [C.POINTER(Options)]
    L.cb_model_create.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(Options), C.POINTER(vp)]
    L.cb_model_destroy.argtypes = [vp]
    L.cb_model_info.argtypes = [vp, C.POINTER(Info)]
    L.cb_last_error.argtypes = [vp]
    L.cb_last_error.restype = C.c_char_p
    L.cb_msal_begin.argtypes = [vp, C.POINTER(Step)]
    L.cb_msal_step.argtypes = [vp, C.POINTER(Step)]
    L.cb_get_displacements.argtypes = [vp, dp, dp]
    L.cb_get_topology.argtypes = [vp, lp, dp]
    L.cb_get_timers.argtypes = [vp, C.POINTER(Timers)]
    L.cb_reset_timers.argtypes = [vp]
    L.cb_set_timing.argtypes = [vp, C.c_int]
    L.cb_set_wait_limit.argtypes = [vp, C.c_longlong]
    L.cb_get_iteration_log.argtypes = [vp, dp, C.c_int, ip]
    L.cb_event_mark.argtypes = [vp, C.c_int]
    L.cb_event_elapsed.argtypes = [vp, C.c_int, C.c_int, dp]
    L.cb_profile_kernel.argtypes = [vp, C.c_int, C.c_int, dp, dp, dp]
    L.cb_eval_forces.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
    L.cb_eval_tangent.argtypes = [vp, dp, dp, dp, dp, lp, dp]
    L.cb_factor_solve.argtypes = [vp, dp, dp, dp, ip]
    L.cb_solve_noalloc.argtypes = [vp, vp, vp]
    L.cb_batch_msal.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.POINTER(Step), ip]
    L.cb_results_open.argtypes = [vp, C.c_char_p]
    L.cb_results_write.argtypes = [vp, C.c_double, C.c_int]
    L.cb_results_close.argtypes = [vp]
    L.cb_input_echo.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]
    L.cb_newton_begin.argtypes = [vp]
    L.cb_newton_step.argtypes = [vp, C.POINTER(Step)]
    L.cb_newmark_begin.argtypes = [vp]
    L.cb_newmark_step.argtypes = [vp, C.POINTER(Step)]
    L.cb_newmark_state.argtypes = [vp, dp, dp, dp]
    L.cb_eval_frame_forces.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
    L.cb_eval_frame_tangent.argtypes = [vp, dp, dp, dp, dp, lp, dp]
    L.cb_eval_frame_mass.argtypes = [vp, dp, dp, dp]
    L.cb_set_krylov_tolerance.argtypes = [vp, C.c_double]
    L.cb_get_krylov_stats.argtypes = [vp, C.POINTER(KrylovStats)]
    fp = C.POINTER(C.c_float)
    L.cb_set_learning.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double]
    L.cb_mpnn_param_count.restype = C.c_long
    L.cb_mpnn_set_params.argtypes = [vp, fp]
    L.cb_mpnn_get_params.argtypes = [vp, fp, fp]
    L.cb_mpnn_eval.argtypes = [vp, dp, dp, dp, C.c_int, dp, dp]
    _lib = L
    return L


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def input_echo(model_def: str) -> str:
    """The input echo the reference writes to results1.txt for this
    model_def (no GPU needed)."""
    text = model_def.encode()
    n = C.c_size_t()
    rc = load().cb_input_echo(text, len(text), None, 0, C.byref(n))
    if rc != 0:
        raise CubensError(rc, "model_def rejected by the parser")
    buf = C.create_string_buffer(n.value + 1)
    load().cb_input_echo(text, len(text), buf, n.value + 1, C.byref(n))
    return buf.raw[:n.value].decode()


def batch_msal(models, steps: int, threads: int = 16):
    """Run the arc-length loop of several Models concurrently (cb_batch_msal):
    returns per model dict(lam, its, res, status)."""
    L = load()
    n = len(models)
    hs = (C.c_void_p * n)(*[m.h for m in models])
    out = (Step * (n * steps))()
    st = (C.c_int * n)()
    rc = L.cb_batch_msal(hs, n, steps, threads, out, st)
    res = []
    for i in range(n):
        recs = [out[i * steps + k] for k in range(steps)]
        recs = [r for r in recs if not r.done]
        res.append(dict(lam=np.array([r.lam for r in recs]), its=np.array([r.iterations for r in recs]),
                        res=np.array([r.residual for r in recs]), status=int(st[i])))
    return rc, res


@dataclass
class StepResult:
    lam: float
    iterations: int
    attempts: int
    residual: float
    dk: float
    done: bool


class Model:
    """A model_def uploaded to the GPU, with its MSAL state (resident API)."""

    def __init__(self, model_def: str, precision: int = FP64, device: int = 0, use_graphs: bool = True,
                 solver: int = SOLVER_BAND, restart: int = 0, maxit: int = 0,
                 precond: int = PRECOND_BLOCK_JACOBI, rtol: float | None = None, factor_kernel: int = 0,
                 band_solve: int = 0):
        L = load()
        opt = Options()
        L.cb_default_options(C.byref(opt))
        opt.precision = precision
        opt.device = device
        opt.use_graphs = 1 if use_graphs else 0
        opt.solver = solver
        opt.krylov_restart = restart
        opt.krylov_maxit = maxit
        opt.precond = precond
        opt.factor_kernel = factor_kernel
        opt.band_solve = band_solve
        h = C.c_void_p()
        raw = model_def.encode()
        rc = L.cb_model_create(raw, len(raw), C.byref(opt), C.byref(h))
        self.h = h
        if rc != CB_OK:
            msg = L.cb_last_error(h).decode() if h else ""
            self.close()
            raise CubensError(rc, msg)
        inf = Info()
        L.cb_model_info(self.h, C.byref(inf))
        self.info = {k: getattr(inf, k) for k, _ in Info._fields_}
        self.neq = inf.neq
        self.nj, self.ne_tr, self.ne_fr, self.ne_sh = inf.nj, inf.ne_tr, inf.ne_fr, inf.ne_sh
        if rtol is not None:
            self._check(L.cb_set_krylov_tolerance(self.h, rtol))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            load().cb_model_destroy(self.h)
        self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != CB_OK:
            raise CubensError(rc, load().cb_last_error(self.h).decode())

    def _step(self, fn) -> StepResult:
        s = Step()
        self._check(fn(self.h, C.byref(s)))
        return StepResult(s.lam, s.iterations, s.attempts, s.residual, s.dk, bool(s.done))

    def begin(self) -> StepResult:
        return self._step(load().cb_msal_begin)

    def step(self) -> StepResult:
        return self._step(load().cb_msal_step)

    def displacements(self):
        d = np.zeros(self.neq)
        lam = C.c_double()
        self._check(load().cb_get_displacements(self.h, _d(d), C.byref(lam)))
        return d, lam.value

    def topology(self):
        jc = np.zeros(self.nj * 7, dtype=np.int64)
        q = np.zeros(self.neq)
        self._check(load().cb_get_topology(self.h, jc.ctypes.data_as(C.POINTER(C.c_long)), _d(q)))
        return jc, q

    def run(self, steps: int, with_d: bool = True):
        """First increment plus steps-1 arc-length increments (the output() records)."""
        lam, its, res, ds = [], [], [], []
        r = self.begin()
        for k in range(steps):
            if k > 0:
                r = self.step()
                if r.done:
                    break
            lam.append(r.lam)
            its.append(r.iterations)
            res.append(r.residual)
            if with_d:
                ds.append(self.displacements()[0])
        return dict(lam=np.array(lam), its=np.array(its), res=np.array(res),
                    d=np.array(ds) if with_d else None)

    # ---- nonlinear Newmark (ALGFLAG 5) ----
    def results_open(self, directory):
        self._check(load().cb_results_open(self.h, str(directory).encode()))

    def results_write(self, lam: float, iterations: int):
        self._check(load().cb_results_write(self.h, lam, iterations))

    def results_close(self):
        self._check(load().cb_results_close(self.h))

    def checkpoint_save(self, path):
        """Newmark: the converged state after the last completed time step,
        bit for bit, to a binary file (checkPoint, misc.c:494-603)."""
        self._check(load().cb_checkpoint_save(self.h, str(path).encode()))

    def checkpoint_load(self, path):
        """Newmark, after newmark_begin: continue from a checkpoint of the
        same model (restartStep, misc.c:605-716)."""
        self._check(load().cb_checkpoint_load(self.h, str(path).encode()))

    def newton_begin(self):
        self._check(load().cb_newton_begin(self.h))

    def newton_step(self) -> StepResult:
        return self._step(load().cb_newton_step)

    def run_newton(self, steps: int = 10_000, with_d: bool = True):
        """Static (modified) Newton-Raphson: lam, its, res, d per converged increment."""
        self.newton_begin()
        lam, its, res, ds = [], [], [], []
        for _ in range(steps):
            r = self.newton_step()
            if r.done:
                break
            lam.append(r.lam)
            its.append(r.iterations)
            res.append(r.residual)
            if with_d:
                ds.append(self.displacements()[0])
        out = {"lam": np.array(lam), "its": np.array(its), "res": np.array(res)}
        if with_d:
            out["d"] = np.array(ds)
        return out

    def newmark_begin(self):
        self._check(load().cb_newmark_begin(self.h))

    def newmark_step(self) -> StepResult:
        return self._step(load().cb_newmark_step)

    def newmark_state(self):
        u, v, a = np.zeros(self.neq), np.zeros(self.neq), np.zeros(self.neq)
        self._check(load().cb_newmark_state(self.h, _d(u), _d(v), _d(a)))
        return u, v, a

    def run_newmark(self, steps: int, with_d: bool = True):
        """The first ``steps`` time steps (k = 0 .. steps-1) from rest."""
        t, its, res, att, ds = [], [], [], [], []
        self.newmark_begin()
        for _ in range(steps):
            r = self.newmark_step()
            if r.done:
                break
            t.append(r.lam)
            its.append(r.iterations)
            res.append(r.residual)
            att.append(r.attempts)
            if with_d:
                ds.append(self.displacements()[0])
        return dict(time=np.array(t), its=np.array(its), res=np.array(res), attempts=np.array(att),
                    d=np.array(ds) if with_d else None)

    # ---- element-level entry points ----
    def eval_frame_forces(self, x_temp, dd, c_ip, ef_ip, len_ip, lref):
        F = self.ne_fr
        c_i, len_i, ef_i, f = np.zeros(9 * F), np.zeros(F), np.zeros(14 * F), np.zeros(self.neq)
        args = [_c64(v) for v in (x_temp, dd, c_ip, ef_ip, len_ip, lref)]
        self._check(load().cb_eval_frame_forces(self.h, *[_d(a) for a in args], _d(c_i), _d(len_i), _d(ef_i),
                                                _d(f)))
        return c_i, len_i, ef_i, f

    def eval_frame_tangent(self, c, ef, length, lref):
        maxa = np.zeros(self.neq + 1, dtype=np.int64)
        ss = np.zeros(self.info["lss"])
        args = [_c64(v) for v in (c, ef, length, lref)]
        self._check(load().cb_eval_frame_tangent(self.h, *[_d(a) for a in args],
                                                 maxa.ctypes.data_as(C.POINTER(C.c_long)), _d(ss)))
        return maxa, ss

    def eval_frame_mass(self, x):
        sm, L = np.zeros(self.neq), np.zeros(self.ne_fr)
        self._check(load().cb_eval_frame_mass(self.h, _d(_c64(x)), _d(sm), _d(L)))
        return sm, L
    def eval_forces(self, x_temp, dd, c_ip=None, ef_ip=None):
        E, T = self.ne_sh, self.ne_tr
        c_i, a_i, ef_i = np.zeros(9 * E), np.zeros(E), np.zeros(18 * E)
        ef_tr, f = np.zeros(2 * T), np.zeros(self.neq)
        args = [_c64(x_temp), _c64(dd), _c64(c_ip) if E else None, _c64(ef_ip) if E else None]
        self._check(load().cb_eval_forces(self.h, *[_d(a) for a in args], _d(c_i), _d(a_i), _d(ef_i),
                                          _d(ef_tr), _d(f)))
        return c_i, a_i, ef_i, ef_tr, f

    def eval_tangent(self, x, c_sh=None, area_sh=None, ef_tr=None):
        maxa = np.zeros(self.neq + 1, dtype=np.int64)
        ss = np.zeros(self.info["lss"])
        args = [_c64(x), _c64(c_sh) if self.ne_sh else None, _c64(area_sh) if self.ne_sh else None,
                _c64(ef_tr) if self.ne_tr else None]
        self._check(load().cb_eval_tangent(self.h, *[_d(a) for a in args],
                                           maxa.ctypes.data_as(C.POINTER(C.c_long)), _d(ss)))
        return maxa, ss

    def factor_solve(self, rhs):
        v = np.zeros(self.neq)
        ssd = np.zeros(self.neq)
        det = C.c_int()
        self._check(load().cb_factor_solve(self.h, _d(_c64(rhs)), _d(v), _d(ssd), C.byref(det)))
        return v, ssd, det.value

    def mark(self, slot: int):
        self._check(load().cb_event_mark(self.h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        v = C.c_double()
        self._check(load().cb_event_elapsed(self.h, a, b, C.byref(v)))
        return v.value

    def profile_kernel(self, which: int, reps: int = 20):
        ms, by, fl = C.c_double(), C.c_double(), C.c_double()
        self._check(load().cb_profile_kernel(self.h, which, reps, C.byref(ms), C.byref(by), C.byref(fl)))
        return ms.value, by.value, fl.value

    def set_learning(self, train_steps: int = -1, adam_per_solve: int = 4, lr: float = 1e-3,
                     stall_factor: float = 2.0):
        self._check(load().cb_set_learning(self.h, train_steps, adam_per_solve, lr, stall_factor))

    def mpnn_params(self):
        L = load()
        n = L.cb_mpnn_param_count()
        th = np.zeros(n, dtype=np.float32)
        gr = np.zeros(n, dtype=np.float32)
        fp = C.POINTER(C.c_float)
        self._check(L.cb_mpnn_get_params(self.h, th.ctypes.data_as(fp), gr.ctypes.data_as(fp)))
        return th, gr

    def set_mpnn_params(self, theta):
        th = np.ascontiguousarray(theta, dtype=np.float32)
        self._check(load().cb_mpnn_set_params(self.h, th.ctypes.data_as(C.POINTER(C.c_float))))

    def mpnn_eval(self, r, p, t=None, train: bool = False):
        """The network on (r, p): z, and with t the loss (gradient via mpnn_params)."""
        z = np.zeros(self.neq)
        loss = C.c_double()
        self._check(load().cb_mpnn_eval(self.h, _d(_c64(r)), _d(_c64(p)), None if t is None else _d(_c64(t)),
                                        1 if train else 0, _d(z), C.byref(loss)))
        return z, loss.value

    def krylov_stats(self) -> dict:
        s = KrylovStats()
        self._check(load().cb_get_krylov_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in KrylovStats._fields_}

    def timers(self) -> dict:
        t = Timers()
        load().cb_get_timers(self.h, C.byref(t))
        return {k: getattr(t, k) for k, _ in Timers._fields_}

    def reset_timers(self):
        load().cb_reset_timers(self.h)

    def set_timing(self, on: bool):
        load().cb_set_timing(self.h, 1 if on else 0)

    def set_wait_limit(self, polls: int):
        """Bound of the persistent kernels' grid-barrier waits (0: the default;
        < 0: a CTA that is not the last to arrive gives up at once)."""
        self._check(load().cb_set_wait_limit(self.h, polls))

    def iteration_log(self):
        """Convergence history of the latest increment: rows (lam, |dd|/|d|,
        |lam q - f|/|lam q|), one per iteration."""
        L = load()
        n = C.c_int()
        self._check(L.cb_get_iteration_log(self.h, None, 0, C.byref(n)))
        out = np.zeros((max(1, n.value), 3))
        self._check(L.cb_get_iteration_log(self.h, _d(out), n.value, C.byref(n)))
        return out[:n.value]
