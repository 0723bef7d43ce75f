"""TEST INFRASTRUCTURE: ctypes front ends of the two CPU checkers.

  RefLib  -- the reference itself (oracle/_ref/libhepem_ref.so, built from the
             reference sources by `make -C oracle ref`; only where those exist)
  PortLib -- the CPU port (oracle/_build/libhepem_port.so, `make -C oracle port`)

Both take numpy arrays and return numpy arrays, with the same call shapes, so
that tests can compare either against the GPU path.  Only tests, the smoke
check and the CPU-baseline leg of bench.py import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_SO = os.path.join(HERE, "_ref", "libhepem_ref.so")
PORT_SO = os.path.join(HERE, "_build", "libhepem_port.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_bp = C.POINTER(C.c_int8)
_ubp = C.POINTER(C.c_uint8)


class TrackState(C.Structure):
    _fields_ = [("type", _bp), ("imc", _ip), ("id", _ip), ("ekin", _dp), ("dir_x", _dp), ("dir_y", _dp),
                ("dir_z", _dp), ("nia0", _dp), ("nia1", _dp), ("nia2", _dp), ("nia3", _dp), ("safety", _dp),
                ("on_boundary", _ubp), ("msc_init_range", _dp), ("msc_dyn_factor", _dp),
                ("msc_tlimit_min", _dp), ("msc_first_step", _ubp), ("gauss_valid", _ubp),
                ("gauss_value", _dp), ("rng_cursor", _ip)]


class StepOut(C.Structure):
    _fields_ = [("edep", _dp), ("gstep", _dp), ("pstep", _dp), ("winner", _bp), ("disp_x", _dp),
                ("disp_y", _dp), ("disp_z", _dp), ("flags", _ubp), ("n_sec", _bp), ("sec_type", _bp),
                ("sec_ekin", _dp), ("sec_dir_x", _dp), ("sec_dir_y", _dp), ("sec_dir_z", _dp)]


STATE_FIELDS = [(f, t) for f, t in [
    ("type", np.int8), ("imc", np.int32), ("id", np.int32), ("ekin", np.float64), ("dir_x", np.float64),
    ("dir_y", np.float64), ("dir_z", np.float64), ("nia0", np.float64), ("nia1", np.float64),
    ("nia2", np.float64), ("nia3", np.float64), ("safety", np.float64), ("on_boundary", np.uint8),
    ("msc_init_range", np.float64), ("msc_dyn_factor", np.float64), ("msc_tlimit_min", np.float64),
    ("msc_first_step", np.uint8), ("gauss_valid", np.uint8), ("gauss_value", np.float64),
    ("rng_cursor", np.int32)]]
OUT_FIELDS = [("edep", np.float64, 1), ("gstep", np.float64, 1), ("pstep", np.float64, 1),
              ("winner", np.int8, 1), ("disp_x", np.float64, 1), ("disp_y", np.float64, 1),
              ("disp_z", np.float64, 1), ("flags", np.uint8, 1), ("n_sec", np.int8, 1),
              ("sec_type", np.int8, 2), ("sec_ekin", np.float64, 2), ("sec_dir_x", np.float64, 2),
              ("sec_dir_y", np.float64, 2), ("sec_dir_z", np.float64, 2)]


def _ptr(a, ct):
    return a.ctypes.data_as(ct)


def _ctype_of(dt):
    return {np.float64: _dp, np.int32: _ip, np.int8: _bp, np.uint8: _ubp}[dt]


def make_state_struct(state: dict) -> TrackState:
    s = TrackState()
    for f, dt in STATE_FIELDS:
        a = state[f]
        assert a.dtype == dt and a.flags.c_contiguous, f
        setattr(s, f, _ptr(a, _ctype_of(dt)))
    return s


def alloc_out(n: int) -> dict:
    return {f: np.zeros(n * k, dtype=dt) for f, dt, k in OUT_FIELDS}


def make_out_struct(out: dict) -> StepOut:
    s = StepOut()
    for f, dt, _ in OUT_FIELDS:
        setattr(s, f, _ptr(out[f], _ctype_of(dt)))
    return s


def copy_state(state: dict) -> dict:
    return {k: v.copy() for k, v in state.items()}


def reference_dir() -> str:
    """Where the reference sources lie: $HEPEM_REFERENCE_DIR, else the
    default of oracle/Makefile (`make print-ref`)."""
    env = os.environ.get("HEPEM_REFERENCE_DIR")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip()


def build_ref(quiet=True) -> bool:
    """Compile oracle/_ref (needs the reference sources)."""
    r = subprocess.run(["make", "-C", HERE, "ref", f"REF={reference_dir()}"], capture_output=quiet)
    return r.returncode == 0 and os.path.exists(REF_SO)


def build_port(quiet=True) -> bool:
    r = subprocess.run(["make", "-C", HERE, "port"], capture_output=quiet)
    return r.returncode == 0 and os.path.exists(PORT_SO)


class _Lib:
    prefix = ""

    def __init__(self, so_path):
        self.lib = C.CDLL(so_path)
        p = self.prefix
        L = self.lib
        getattr(L, p + "load_state").restype = C.c_void_p
        getattr(L, p + "load_state").argtypes = [C.c_char_p]
        getattr(L, p + "free_state").argtypes = [C.c_void_p]
        getattr(L, p + "electron_lookup").argtypes = [C.c_void_p, C.c_int64, C.c_int, _dp, _ip] + [_dp] * 5
        getattr(L, p + "step").argtypes = [C.c_void_p, C.c_int64, C.POINTER(TrackState), C.POINTER(TrackState),
                                           _dp, C.c_int32, C.c_uint64, C.POINTER(StepOut)]
        getattr(L, p + "step").restype = C.c_int
        getattr(L, p + "electron_xs_stepping").argtypes = [C.c_void_p, C.c_int64, C.c_int, _dp, _ip] + [_dp] * 5
        getattr(L, p + "brem_select_target").argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, _dp, _ip, _dp,
                                                         _ip]
        getattr(L, p + "gamma_xs").argtypes = [C.c_void_p, C.c_int64, _dp, _ip, _dp, _dp, _dp, _ip]
        getattr(L, p + "conv_select_target").argtypes = [C.c_void_p, C.c_int64, _dp, _ip, _dp, _ip]
        getattr(L, p + "step_geom").argtypes = [C.c_void_p, C.c_int64, C.POINTER(TrackState),
                                                C.POINTER(TrackState), _dp, C.c_int32, C.c_uint64, _dp, _dp,
                                                _dp, _dp, _ubp, _dp, C.POINTER(StepOut)]
        getattr(L, p + "step_geom").restype = C.c_int
        self.st = None

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    def load(self, json_path: str):
        self.st = self._f("load_state")(json_path.encode())
        if not self.st:
            raise RuntimeError(f"could not load state {json_path}")
        return self

    def close(self):
        if self.st:
            self._f("free_state")(self.st)
            self.st = None

    def electron_lookup(self, ekin, imc, positron=False):
        n = len(ekin)
        ekin = np.ascontiguousarray(ekin, dtype=np.float64)
        imc = np.ascontiguousarray(imc, dtype=np.int32)
        outs = [np.empty(n) for _ in range(5)]
        self._f("electron_lookup")(self.st, n, int(positron), _ptr(ekin, _dp), _ptr(imc, _ip),
                                   *[_ptr(o, _dp) for o in outs])
        return dict(zip(["xs_ioni", "xs_brem", "dedx", "range", "invrange_half"], outs))

    def electron_xs_stepping(self, ekin, imc, positron=False):
        n = len(ekin)
        ekin = np.ascontiguousarray(ekin, dtype=np.float64)
        imc = np.ascontiguousarray(imc, dtype=np.int32)
        outs = [np.empty(n) for _ in range(5)]
        self._f("electron_xs_stepping")(self.st, n, int(positron), _ptr(ekin, _dp), _ptr(imc, _ip),
                                        *[_ptr(o, _dp) for o in outs])
        return dict(zip(["xs_ioni", "xs_brem", "xs_annih", "xs_nuc", "tr_mfp"], outs))

    def brem_select_target(self, ekin, imc, urnd, positron=False, sb=True):
        n = len(ekin)
        ekin = np.ascontiguousarray(ekin, dtype=np.float64)
        imc = np.ascontiguousarray(imc, dtype=np.int32)
        urnd = np.ascontiguousarray(urnd, dtype=np.float64)
        out = np.empty(n, dtype=np.int32)
        self._f("brem_select_target")(self.st, n, int(positron), int(sb), _ptr(ekin, _dp), _ptr(imc, _ip),
                                      _ptr(urnd, _dp), _ptr(out, _ip))
        return out

    def gamma_xs(self, ekin, imc, urnd):
        n = len(ekin)
        ekin = np.ascontiguousarray(ekin, dtype=np.float64)
        imc = np.ascontiguousarray(imc, dtype=np.int32)
        urnd = np.ascontiguousarray(urnd, dtype=np.float64)
        tot, pe = np.empty(n), np.empty(n)
        win = np.empty(n, dtype=np.int32)
        self._f("gamma_xs")(self.st, n, _ptr(ekin, _dp), _ptr(imc, _ip), _ptr(urnd, _dp), _ptr(tot, _dp),
                            _ptr(pe, _dp), _ptr(win, _ip))
        return dict(xs_tot=tot, xs_pe=pe, winner=win)

    def conv_select_target(self, ekin, imc, urnd):
        n = len(ekin)
        ekin = np.ascontiguousarray(ekin, dtype=np.float64)
        imc = np.ascontiguousarray(imc, dtype=np.int32)
        urnd = np.ascontiguousarray(urnd, dtype=np.float64)
        out = np.empty(n, dtype=np.int32)
        self._f("conv_select_target")(self.st, n, _ptr(ekin, _dp), _ptr(imc, _ip), _ptr(urnd, _dp),
                                      _ptr(out, _ip))
        return out

    def step(self, state: dict, uniforms: np.ndarray, n_uniform: int, seed: int, in_place=False):
        n = len(state["ekin"])
        out_state = state if in_place else copy_state(state)
        res = alloc_out(n)
        sin = make_state_struct(state)
        sout = make_state_struct(out_state)
        sres = make_out_struct(res)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        rc = self._f("step")(self.st, n, C.byref(sin), C.byref(sout), _ptr(u, _dp), n_uniform, seed,
                             C.byref(sres))
        if rc != 0:
            raise RuntimeError(f"step failed rc={rc}")
        return out_state, res


    def step_geom(self, state: dict, uniforms, n_uniform, seed, gfrac, new_dir, post_boundary):
        """HowFar, then a caller's transport -- geometrical step gfrac times the
        proposed one, direction new_dir = (x, y, z) arrays, post-step boundary
        status -- then Perform.  Returns (out_state, res, proposed)."""
        n = len(state["ekin"])
        out_state = copy_state(state)
        res = alloc_out(n)
        gfrac = np.ascontiguousarray(gfrac, dtype=np.float64)
        nd = [np.ascontiguousarray(a, dtype=np.float64) for a in new_dir]
        post = np.ascontiguousarray(post_boundary, dtype=np.uint8)
        proposed = np.empty(n)
        sin, sout, sres = make_state_struct(state), make_state_struct(out_state), make_out_struct(res)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        rc = self._f("step_geom")(self.st, n, C.byref(sin), C.byref(sout), _ptr(u, _dp), n_uniform, seed,
                                  _ptr(gfrac, _dp), *[_ptr(a, _dp) for a in nd], _ptr(post, _ubp),
                                  _ptr(proposed, _dp), C.byref(sres))
        if rc != 0:
            raise RuntimeError(f"step failed rc={rc}")
        return out_state, res, proposed


class RefLib(_Lib):
    prefix = "ref_"

    def __init__(self, so_path=REF_SO):
        super().__init__(so_path)
        L = self.lib
        L.ref_vdt_log.argtypes = [C.c_int64, _dp, _dp]
        L.ref_vdt_exp.argtypes = [C.c_int64, _dp, _dp]
        L.ref_vdt_pow.argtypes = [C.c_int64, _dp, _dp, _dp]
        L.ref_num_couples.argtypes = [C.c_void_p]

    def vdt_log(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self.lib.ref_vdt_log(len(x), _ptr(x, _dp), _ptr(y, _dp))
        return y

    def vdt_exp(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self.lib.ref_vdt_exp(len(x), _ptr(x, _dp), _ptr(y, _dp))
        return y

class PortLib(_Lib):
    prefix = "port_"

    def __init__(self, so_path=PORT_SO):
        super().__init__(so_path)
        L = self.lib
        L.port_step_mt.argtypes = [C.c_void_p, C.c_int64, C.POINTER(TrackState), C.POINTER(TrackState),
                                   _dp, C.c_int32, C.c_uint64, C.POINTER(StepOut), C.c_int]
        L.port_step_mt.restype = C.c_int
        L.port_philox_uniform.argtypes = [C.c_uint64, C.c_int32, C.c_int32]
        L.port_philox_uniform.restype = C.c_double
        L.port_fill_uniforms.argtypes = [C.c_int64, _ip, C.c_int32, C.c_uint64, _dp]
        L.port_vdt_log.argtypes = [C.c_int64, _dp, _dp]
        L.port_vdt_exp.argtypes = [C.c_int64, _dp, _dp]
        L.port_woodcock_gamma.argtypes = [C.c_void_p, C.c_int64, C.POINTER(TrackState), C.POINTER(TrackState),
                                          _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, C.c_int, _dp, _ip,
                                          C.c_double, _dp, C.c_int32, C.c_uint64, C.POINTER(StepOut),
                                          C.POINTER(C.c_uint8)]
        L.port_woodcock_gamma.restype = C.c_int

    def woodcock_gamma(self, state: dict, pos, box: dict, uniforms, n_uniform, seed):
        """Woodcock gamma step in a layered box (restatement of the reference
        helper's loop); pos = (x, y, z) arrays, updated copies are returned."""
        n = len(state["ekin"])
        out_state = copy_state(state)
        res = alloc_out(n)
        px, py, pz = (np.array(a, dtype=np.float64, copy=True) for a in pos)
        reached = np.zeros(n, dtype=np.uint8)
        zb = np.ascontiguousarray(box["z_bounds"], dtype=np.float64)
        li = np.ascontiguousarray(box["layer_imc"], dtype=np.int32)
        sin, sout, sres = make_state_struct(state), make_state_struct(out_state), make_out_struct(res)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        rc = self.lib.port_woodcock_gamma(self.st, n, C.byref(sin), C.byref(sout), _ptr(px, _dp), _ptr(py, _dp),
                                          _ptr(pz, _dp), box["half_x"], box["half_y"], len(li), box["wdt_imc"],
                                          _ptr(zb, _dp), _ptr(li, _ip), box["energy_limit"], _ptr(u, _dp),
                                          n_uniform, seed, C.byref(sres),
                                          reached.ctypes.data_as(C.POINTER(C.c_uint8)))
        if rc != 0:
            raise RuntimeError(f"woodcock failed rc={rc}")
        return out_state, res, (px, py, pz), reached

    def step_mt(self, state: dict, uniforms, n_uniform, seed, threads, in_place=False):
        n = len(state["ekin"])
        out_state = state if in_place else copy_state(state)
        res = alloc_out(n)
        sin, sout, sres = make_state_struct(state), make_state_struct(out_state), make_out_struct(res)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        rc = self.lib.port_step_mt(self.st, n, C.byref(sin), C.byref(sout), _ptr(u, _dp), n_uniform, seed,
                                   C.byref(sres), threads)
        if rc != 0:
            raise RuntimeError(f"step failed rc={rc}")
        return out_state, res

    def step_mt_fn(self, state: dict, out_state: dict, res: dict, uniforms, n_uniform, seed, threads):
        """A function of no arguments that steps `state` into `out_state` and
        `res` on `threads` host threads; the argument structs are built once,
        so a timing loop times the port's step alone."""
        n = len(state["ekin"])
        sin, sout, sres = make_state_struct(state), make_state_struct(out_state), make_out_struct(res)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        up = _ptr(u, _dp)

        def run():
            rc = self.lib.port_step_mt(self.st, n, C.byref(sin), C.byref(sout), up, n_uniform, seed,
                                       C.byref(sres), threads)
            if rc != 0:
                raise RuntimeError(f"step failed rc={rc}")

        run.keep = (state, out_state, res, u, sin, sout, sres)  # the arrays stay alive with the function
        return run

    def fill_uniforms(self, ids, n_uniform, seed):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        u = np.empty(len(ids) * n_uniform)
        self.lib.port_fill_uniforms(len(ids), _ptr(ids, _ip), n_uniform, seed, _ptr(u, _dp))
        return u

    def vdt_log(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self.lib.port_vdt_log(len(x), _ptr(x, _dp), _ptr(y, _dp))
        return y

    def vdt_exp(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self.lib.port_vdt_exp(len(x), _ptr(x, _dp), _ptr(y, _dp))
        return y
