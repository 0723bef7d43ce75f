"""ctypes front end of libg4hepem_gb300.so (the C-ABI of include/g4hepem_gb300.h).

Device memory and streams come from torch; the library takes raw pointers.
Importing this module never falls back to anything: if the library is missing
it raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libg4hepem_gb300.so")

_vp = C.c_void_p

STATE_FIELDS = [("type", np.int8), ("imc", np.int32), ("id", np.int32), ("ekin", np.float64),
                ("dir_x", np.float64), ("dir_y", np.float64), ("dir_z", np.float64), ("nia0", np.float64),
                ("nia1", np.float64), ("nia2", np.float64), ("nia3", np.float64), ("safety", np.float64),
                ("on_boundary", np.uint8), ("msc_init_range", np.float64), ("msc_dyn_factor", np.float64),
                ("msc_tlimit_min", np.float64), ("msc_first_step", np.uint8), ("gauss_valid", np.uint8),
                ("gauss_value", np.float64), ("rng_cursor", np.int32)]
# (name, dtype, slots per track)
OUT_FIELDS = [("edep", np.float64, 1), ("gstep", np.float64, 1), ("pstep", np.float64, 1), ("winner", np.int8, 1),
              ("disp_x", np.float64, 1), ("disp_y", np.float64, 1), ("disp_z", np.float64, 1),
              ("flags", np.uint8, 1), ("n_sec", np.int8, 1), ("sec_type", np.int8, 2),
              ("sec_ekin", np.float64, 2), ("sec_dir_x", np.float64, 2), ("sec_dir_y", np.float64, 2),
              ("sec_dir_z", np.float64, 2)]
# fields copied back by hepem_step_host (persistent outputs of the step)
STATE_OUT_FIELDS = [f for f, _ in STATE_FIELDS if f not in ("type", "imc", "id", "safety", "on_boundary")]

FLAG_RNG_OVERFLOW, FLAG_LOOP_CAP, FLAG_BAD_INPUT, FLAG_BAD_INDEX = 1, 2, 4, 8
NOALLOC_MAX_TRACKS = 524288  # HEPEM_NOALLOC_MAX_TRACKS


class TrackState(C.Structure):
    _fields_ = [(f, _vp) for f, _ in STATE_FIELDS]


class StepOut(C.Structure):
    _fields_ = [(f, _vp) for f, _, _ in OUT_FIELDS]


class StepCounters(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("uniforms", C.c_uint64), ("rng_overflow", C.c_uint64),
                ("secondaries", C.c_uint64), ("interactions", C.c_uint64 * 8), ("fp64_fallback", C.c_uint64)]


class SubBatch(C.Structure):
    _fields_ = [("offset", C.c_int64), ("n", C.c_int64), ("seed", C.c_uint64)]


class LaunchConfig(C.Structure):
    _fields_ = [("block", C.c_int32 * 11), ("ctas_per_sm", C.c_int32 * 11), ("sort_energy_bins", C.c_int32),
                ("ms", C.c_float * 11)]

    def as_dict(self) -> dict:
        return {"block": list(self.block), "ctas_per_sm": list(self.ctas_per_sm),
                "sort_energy_bins": self.sort_energy_bins, "ms": [round(x, 4) for x in self.ms]}


class LayeredBox(C.Structure):
    _fields_ = [("half_x", C.c_double), ("half_y", C.c_double), ("n_layers", C.c_int32), ("wdt_imc", C.c_int32),
                ("z_bounds", _vp), ("layer_imc", _vp), ("energy_limit", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_int64), ("max_steps", C.c_int32), ("max_requests", C.c_int32),
                ("min_energy", C.c_double), ("precision", C.c_int32), ("reserved", C.c_int32)]


class RequestResult(C.Structure):
    _fields_ = [("n_tracks", C.c_int64), ("steps", C.c_int32), ("status", C.c_int32), ("edep", C.c_double),
                ("e_secondaries", C.c_double), ("n_secondaries", C.c_int64), ("track_steps", C.c_int64),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerStats(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("track_steps", C.c_int64), ("completed", C.c_int64),
                ("waiting", C.c_int64), ("active", C.c_int64), ("free_slots", C.c_int64),
                ("batch_ms_p50", C.c_double), ("batch_ms_p99", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


EXPORTED = ["hepem_create", "hepem_create_from_file", "hepem_image_from_json", "hepem_image_check",
            "hepem_create_from_image", "hepem_destroy", "hepem_info", "hepem_status_string",
            "hepem_last_error", "hepem_electron_lookup", "hepem_electron_lookup_mixed", "hepem_step", "hepem_step_batched",
            "hepem_step_batched_noalloc", "hepem_step_mixed", "hepem_step_host", "hepem_step_host_mixed",
            "hepem_philox_uniform", "hepem_fill_uniforms", "hepem_profile_stages", "hepem_stage_times",
            "hepem_server_create", "hepem_server_capacity", "hepem_server_submit", "hepem_server_poll",
            "hepem_server_wait", "hepem_server_cancel", "hepem_server_get_stats", "hepem_server_reset_stats",
            "hepem_server_destroy", "hepem_sample_model", "hepem_stack_secondaries", "hepem_woodcock_gamma", "hepem_get_launch_config", "hepem_set_launch_config", "hepem_autotune",
            "hepem_set_table_l2_window", "hepem_step_limit_bytes", "hepem_howfar", "hepem_perform",
            "hepem_howfar_host", "hepem_perform_host", "hepem_electron_xs_stepping", "hepem_brem_select_target",
            "hepem_conv_select_target", "hepem_gamma_xs", "hepem_step_subbatches", "hepem_server_snapshot",
            "hepem_server_snapshot_check", "hepem_server_resume"]
FORMS = {"plain": 0, "batched": 1, "mixed": 2}
STATUS_CANCELLED, STATUS_TIMEOUT, STATUS_OOM_ADMISSION = 8, 5, 6


class HepEmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run g4hepem_gb300.build.build() first")
        L = C.CDLL(LIB_PATH)
        L.hepem_create.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(_vp)]
        L.hepem_create_from_file.argtypes = [C.c_char_p, C.POINTER(_vp)]
        L.hepem_destroy.argtypes = [_vp]
        L.hepem_image_from_json.argtypes = [C.c_char_p, C.c_size_t, _vp, C.c_size_t, C.POINTER(C.c_size_t)]
        L.hepem_image_check.argtypes = [_vp, C.c_size_t, C.POINTER(C.c_int64)]
        L.hepem_create_from_image.argtypes = [_vp, C.c_size_t, C.POINTER(_vp)]
        L.hepem_info.argtypes = [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int64)]
        L.hepem_status_string.argtypes = [C.c_int]
        L.hepem_status_string.restype = C.c_char_p
        L.hepem_last_error.restype = C.c_char_p
        L.hepem_electron_lookup.argtypes = [_vp, C.c_int64, C.c_int] + [_vp] * 7 + [_vp]
        L.hepem_electron_lookup_mixed.argtypes = L.hepem_electron_lookup.argtypes
        L.hepem_step.argtypes = [_vp, C.c_int64, C.POINTER(TrackState), C.POINTER(TrackState), _vp, C.c_int32,
                                 C.c_uint64, C.POINTER(StepOut), _vp, _vp]
        L.hepem_step_host.argtypes = L.hepem_step.argtypes
        L.hepem_step_host_mixed.argtypes = L.hepem_step.argtypes
        L.hepem_step_batched.argtypes = L.hepem_step.argtypes
        L.hepem_step_batched_noalloc.argtypes = L.hepem_step.argtypes
        L.hepem_step_mixed.argtypes = L.hepem_step.argtypes
        L.hepem_woodcock_gamma.argtypes = [_vp, C.c_int64, C.POINTER(TrackState), C.POINTER(TrackState), _vp, _vp,
                                           _vp, C.POINTER(LayeredBox), _vp, C.c_int32, C.c_uint64,
                                           C.POINTER(StepOut), _vp, _vp]
        L.hepem_stack_secondaries.argtypes = [_vp, C.c_int64, C.POINTER(TrackState), C.POINTER(StepOut), C.c_int,
                                              C.c_int32, C.POINTER(TrackState), C.c_int64, _vp, _vp, _vp]
        L.hepem_sample_model.argtypes = [_vp, C.c_int, C.c_int, C.c_int64, C.c_double, C.c_int32, C.c_uint64, _vp,
                                         _vp, _vp]
        L.hepem_philox_uniform.argtypes = [C.c_uint64, C.c_int32, C.c_int32]
        L.hepem_philox_uniform.restype = C.c_double
        L.hepem_fill_uniforms.argtypes = [C.c_int64, _vp, C.c_int32, C.c_uint64, _vp, _vp]
        L.hepem_profile_stages.argtypes = [_vp, C.c_int]
        L.hepem_stage_times.argtypes = [_vp, C.POINTER(C.c_float), C.POINTER(C.c_char_p), C.c_int32,
                                        C.POINTER(C.c_int32)]
        L.hepem_get_launch_config.argtypes = [_vp, C.POINTER(LaunchConfig)]
        L.hepem_set_launch_config.argtypes = [_vp, C.POINTER(LaunchConfig)]
        L.hepem_set_table_l2_window.argtypes = [_vp, C.c_int, C.POINTER(C.c_int64)]
        L.hepem_autotune.argtypes = [_vp, C.c_int64, C.POINTER(TrackState), _vp, C.c_int32, C.c_uint64, C.c_int,
                                     C.POINTER(LaunchConfig), _vp]
        L.hepem_step_limit_bytes.argtypes = [C.c_int64]
        L.hepem_step_limit_bytes.restype = C.c_int64
        L.hepem_howfar.argtypes = [_vp, C.c_int, C.c_int64, C.POINTER(TrackState), _vp, C.c_int32, C.c_uint64,
                                   _vp, _vp, _vp, _vp]
        L.hepem_howfar_host.argtypes = L.hepem_howfar.argtypes
        L.hepem_perform.argtypes = [_vp, C.c_int, C.c_int64, C.POINTER(TrackState), C.POINTER(TrackState), _vp,
                                    _vp, _vp, C.c_int32, C.c_uint64, C.POINTER(StepOut), _vp, _vp]
        L.hepem_perform_host.argtypes = L.hepem_perform.argtypes
        L.hepem_step_subbatches.argtypes = [_vp, C.c_int, C.c_int32, C.POINTER(SubBatch), C.POINTER(TrackState),
                                            C.POINTER(TrackState), _vp, C.c_int32, C.POINTER(StepOut), _vp, _vp]
        L.hepem_electron_xs_stepping.argtypes = [_vp, C.c_int64, C.c_int, C.c_int] + [_vp] * 7 + [_vp]
        L.hepem_brem_select_target.argtypes = [_vp, C.c_int64, C.c_int, C.c_int, C.c_int] + [_vp] * 4 + [_vp]
        L.hepem_conv_select_target.argtypes = [_vp, C.c_int64, C.c_int] + [_vp] * 4 + [_vp]
        L.hepem_gamma_xs.argtypes = [_vp, C.c_int64, C.c_int] + [_vp] * 6 + [_vp]
        L.hepem_server_create.argtypes = [_vp, C.POINTER(ServerConfig), C.POINTER(_vp)]
        L.hepem_server_capacity.argtypes = [_vp, C.POINTER(C.c_int64)]
        L.hepem_server_submit.argtypes = [_vp, C.c_int64, C.POINTER(TrackState), C.c_uint64, C.POINTER(C.c_int64)]
        L.hepem_server_poll.argtypes = [_vp, C.c_int64, C.POINTER(C.c_int32), C.POINTER(RequestResult),
                                        C.POINTER(TrackState)]
        L.hepem_server_wait.argtypes = [_vp, C.c_int64, C.c_double, C.POINTER(RequestResult),
                                        C.POINTER(TrackState)]
        L.hepem_server_cancel.argtypes = [_vp, C.c_int64]
        L.hepem_server_get_stats.argtypes = [_vp, C.POINTER(ServerStats)]
        L.hepem_server_reset_stats.argtypes = [_vp]
        L.hepem_server_destroy.argtypes = [_vp]
        L.hepem_server_snapshot.argtypes = [_vp, _vp, C.c_size_t, C.POINTER(C.c_size_t)]
        L.hepem_server_snapshot_check.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_int64),
                                                  C.POINTER(C.c_int64)]
        L.hepem_server_resume.argtypes = [_vp, C.c_char_p, C.c_size_t, C.c_int64, C.POINTER(C.c_int64),
                                          C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        _LIB = L
    return _LIB


def check(rc):
    if rc != 0:
        L = lib()
        raise HepEmError(rc, f"{L.hepem_status_string(rc).decode()}: {L.hepem_last_error().decode()}")


def _ptr(x):
    """Raw data pointer of a torch tensor or numpy array (None: a null pointer)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


def _stream_ptr(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def make_state_struct(arrs: dict) -> TrackState:
    s = TrackState()
    for f, _ in STATE_FIELDS:
        setattr(s, f, _ptr(arrs[f]))
    return s


def make_out_struct(arrs: dict) -> StepOut:
    s = StepOut()
    for f, _, _ in OUT_FIELDS:
        setattr(s, f, _ptr(arrs[f]))
    return s


class Context:
    """Tables of one G4HepEmState on the current CUDA device."""

    def __init__(self, json_path: str | None = None, json_text: str | bytes | None = None,
                 image: bytes | None = None):
        L = lib()
        h = _vp()
        if image is not None:
            check(L.hepem_create_from_image(image, len(image), C.byref(h)))
        elif json_text is not None:
            b = json_text.encode() if isinstance(json_text, str) else json_text
            check(L.hepem_create(b, len(b), C.byref(h)))
        else:
            check(L.hepem_create_from_file(json_path.encode(), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().hepem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        nc, nm, nr, nb = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int64()
        check(lib().hepem_info(self.h, C.byref(nc), C.byref(nm), C.byref(nr), C.byref(nb)))
        return dict(n_couples=nc.value, n_materials=nm.value, n_regions=nr.value, arena_bytes=nb.value)

    # -- device-pointer entry points (torch CUDA tensors) ----------------------
    def electron_lookup(self, ekin, imc, positron=False, out=None, stream=None, mixed=False):
        """hepem_electron_lookup (FP64), or with mixed=True hepem_electron_lookup_mixed (FP32 tables)."""
        import torch
        n = ekin.numel()
        if out is None:
            out = {k: torch.empty(n, dtype=torch.float64, device=ekin.device)
                   for k in ("xs_ioni", "xs_brem", "dedx", "range", "invrange_half")}
        fn = lib().hepem_electron_lookup_mixed if mixed else lib().hepem_electron_lookup
        check(fn(self.h, n, int(positron), _ptr(ekin), _ptr(imc), _ptr(out["xs_ioni"]),
                                          _ptr(out["xs_brem"]), _ptr(out["dedx"]), _ptr(out["range"]),
                                          _ptr(out["invrange_half"]), _stream_ptr(stream)))
        return out

    def step(self, state_in: dict, state_out: dict, uniforms, n_uniform: int, seed: int, res: dict,
             counters=None, stream=None, form="plain"):
        """One step of every track; form: "plain" (hepem_step), "batched" (hepem_step_batched),
        "mixed" (hepem_step_mixed, the precision form) or "noalloc" (hepem_step_batched_noalloc)."""
        n = state_in["ekin"].numel()
        sin, sout, sres = make_state_struct(state_in), make_state_struct(state_out), make_out_struct(res)
        fn = {"plain": lib().hepem_step, "batched": lib().hepem_step_batched, "mixed": lib().hepem_step_mixed,
              "noalloc": lib().hepem_step_batched_noalloc}[form]
        check(fn(self.h, n, C.byref(sin), C.byref(sout), _ptr(uniforms), n_uniform, seed, C.byref(sres),
                 _ptr(counters) if counters is not None else None, _stream_ptr(stream)))

    def step_subbatches(self, batches, state_in: dict, state_out: dict, uniforms, n_uniform: int, res: dict,
                        counters=None, stream=None, form="batched"):
        """hepem_step_subbatches: batches = [(offset, n, seed), ...] over the same arrays."""
        arr = (SubBatch * max(len(batches), 1))(*[SubBatch(int(o), int(n), int(sd)) for o, n, sd in batches])
        sin, sout, sres = make_state_struct(state_in), make_state_struct(state_out), make_out_struct(res)
        check(lib().hepem_step_subbatches(self.h, FORMS[form], len(batches), arr, C.byref(sin), C.byref(sout),
                                          _ptr(uniforms) if n_uniform else None, n_uniform, C.byref(sres),
                                          _ptr(counters) if counters is not None else None, _stream_ptr(stream)))

    # -- single functions of the path (the reference's device-test quantities) ----
    def electron_xs_stepping(self, ekin, imc, positron=False, mixed=False, stream=None):
        import torch
        n = ekin.numel()
        out = {k: torch.empty(n, dtype=torch.float64, device=ekin.device)
               for k in ("xs_ioni", "xs_brem", "xs_annih", "xs_nuc", "tr_mfp")}
        check(lib().hepem_electron_xs_stepping(self.h, n, int(positron), int(mixed), _ptr(ekin), _ptr(imc),
                                               *[_ptr(v) for v in out.values()], _stream_ptr(stream)))
        return out

    def brem_select_target(self, ekin, imc, urnd, positron=False, sb=True, mixed=False, stream=None):
        import torch
        out = torch.empty(ekin.numel(), dtype=torch.int32, device=ekin.device)
        check(lib().hepem_brem_select_target(self.h, ekin.numel(), int(positron), int(sb), int(mixed), _ptr(ekin),
                                             _ptr(imc), _ptr(urnd), _ptr(out), _stream_ptr(stream)))
        return out

    def conv_select_target(self, ekin, imc, urnd, mixed=False, stream=None):
        import torch
        out = torch.empty(ekin.numel(), dtype=torch.int32, device=ekin.device)
        check(lib().hepem_conv_select_target(self.h, ekin.numel(), int(mixed), _ptr(ekin), _ptr(imc), _ptr(urnd),
                                             _ptr(out), _stream_ptr(stream)))
        return out

    def gamma_xs(self, ekin, imc, urnd, mixed=False, stream=None):
        import torch
        n = ekin.numel()
        tot = torch.empty(n, dtype=torch.float64, device=ekin.device)
        pe = torch.empty(n, dtype=torch.float64, device=ekin.device)
        win = torch.empty(n, dtype=torch.int32, device=ekin.device)
        check(lib().hepem_gamma_xs(self.h, n, int(mixed), _ptr(ekin), _ptr(imc), _ptr(urnd), _ptr(tot), _ptr(pe),
                                   _ptr(win), _stream_ptr(stream)))
        return dict(xs_tot=tot, xs_pe=pe, winner=win)

    # -- HowFar and Perform as two calls (the caller's transport between them) -----
    def howfar(self, state: dict, uniforms, n_uniform: int, seed: int, gstep=None, limits=None, counters=None,
               stream=None, form="plain"):
        """hepem_howfar on device tensors: returns (gstep, limits), the proposed
        geometrical steps and the step-limit record for perform()."""
        import torch
        n = state["ekin"].numel()
        if gstep is None:
            gstep = torch.empty(n, dtype=torch.float64, device=state["ekin"].device)
        if limits is None:
            limits = torch.empty(max(int(lib().hepem_step_limit_bytes(n)), 1), dtype=torch.uint8,
                                 device=state["ekin"].device)
        sin = make_state_struct(state)
        check(lib().hepem_howfar(self.h, FORMS[form], n, C.byref(sin), _ptr(uniforms) if n_uniform else None,
                                 n_uniform, seed, _ptr(gstep), _ptr(limits),
                                 _ptr(counters) if counters is not None else None, _stream_ptr(stream)))
        return gstep, limits

    def perform(self, state_in: dict, state_out: dict, gstep, limits, uniforms, n_uniform: int, seed: int,
                res: dict, counters=None, stream=None, form="plain"):
        """hepem_perform on device tensors (state_in carries the direction and
        boundary status after transport; gstep the steps made)."""
        n = state_in["ekin"].numel()
        sin, sout, sres = make_state_struct(state_in), make_state_struct(state_out), make_out_struct(res)
        check(lib().hepem_perform(self.h, FORMS[form], n, C.byref(sin), C.byref(sout), _ptr(gstep), _ptr(limits),
                                  _ptr(uniforms) if n_uniform else None, n_uniform, seed, C.byref(sres),
                                  _ptr(counters) if counters is not None else None, _stream_ptr(stream)))

    def howfar_host(self, state: dict, uniforms, n_uniform: int, seed: int, form="plain", stream=None):
        """hepem_howfar_host on numpy arrays: returns (gstep, limits, counters)."""
        n = len(state["ekin"])
        gstep = np.empty(n)
        limits = np.empty(max(int(lib().hepem_step_limit_bytes(n)), 1), dtype=np.uint8)
        cnt = StepCounters()
        sin = make_state_struct(state)
        check(lib().hepem_howfar_host(self.h, FORMS[form], n, C.byref(sin), _ptr(uniforms) if n_uniform else None,
                                      n_uniform, seed, _ptr(gstep), _ptr(limits), C.byref(cnt),
                                      _stream_ptr(stream)))
        return gstep, limits, cnt

    def perform_host(self, state_in: dict, state_out: dict, gstep, limits, uniforms, n_uniform: int, seed: int,
                     res: dict, form="plain", stream=None):
        """hepem_perform_host on numpy arrays; returns the counters."""
        n = len(state_in["ekin"])
        cnt = StepCounters()
        sin, sout, sres = make_state_struct(state_in), make_state_struct(state_out), make_out_struct(res)
        check(lib().hepem_perform_host(self.h, FORMS[form], n, C.byref(sin), C.byref(sout), _ptr(gstep),
                                       _ptr(limits), _ptr(uniforms) if n_uniform else None, n_uniform, seed,
                                       C.byref(sres), C.byref(cnt), _stream_ptr(stream)))
        return cnt

    # -- Woodcock gamma tracking ---------------------------------------------------
    def woodcock_gamma(self, state_in: dict, state_out: dict, pos: tuple, box: dict, uniforms, n_uniform: int,
                       seed: int, res: dict, reached=None, stream=None):
        """hepem_woodcock_gamma; pos = (x, y, z) device arrays (updated in place);
        box: half_x, half_y, z_bounds (device), layer_imc (device), wdt_imc, energy_limit."""
        n = state_in["ekin"].numel()
        b = LayeredBox(box["half_x"], box["half_y"], box["layer_imc"].numel(), box["wdt_imc"],
                       _ptr(box["z_bounds"]), _ptr(box["layer_imc"]), box["energy_limit"])
        sin, sout, sres = make_state_struct(state_in), make_state_struct(state_out), make_out_struct(res)
        check(lib().hepem_woodcock_gamma(self.h, n, C.byref(sin), C.byref(sout), _ptr(pos[0]), _ptr(pos[1]),
                                         _ptr(pos[2]), C.byref(b), _ptr(uniforms) if n_uniform else None,
                                         n_uniform, seed, C.byref(sres),
                                         _ptr(reached) if reached is not None else None, _stream_ptr(stream)))

    # -- secondary stacking ------------------------------------------------------
    def stack_secondaries(self, parents: dict, res: dict, apply_cuts: bool, id_base: int, capacity: int,
                          out: dict | None = None, edep_cut=None, stream=None):
        """hepem_stack_secondaries: returns (new track batch dict, number stacked)."""
        import torch
        n = parents["ekin"].numel()
        if out is None:
            out = empty_state_torch(max(capacity, 1))
        n_out = torch.zeros(1, dtype=torch.int64, device="cuda")
        sp, so, sr = make_state_struct(parents), make_state_struct(out), make_out_struct(res)
        check(lib().hepem_stack_secondaries(self.h, n, C.byref(sp), C.byref(sr), int(apply_cuts), id_base,
                                            C.byref(so), capacity, _ptr(n_out),
                                            _ptr(edep_cut) if edep_cut is not None else None, _stream_ptr(stream)))
        return out, n_out

    # -- per-model sampling -------------------------------------------------------
    SAMPLE_MODELS = {"sb": 0, "rb": 1, "moller": 2, "bhabha": 3, "compton": 4, "conversion": 5}

    def sample_model(self, model: str, n: int, ekin: float, imc: int, seed: int, mixed=False, out=None,
                     stream=None):
        """n draws of one interaction model (hepem_sample_model); returns (energies, fallback count)."""
        import torch
        if out is None:
            out = torch.empty(n, dtype=torch.float64, device="cuda")
        fb = torch.zeros(1, dtype=torch.int64, device="cuda")
        check(lib().hepem_sample_model(self.h, self.SAMPLE_MODELS[model], int(mixed), n, ekin, imc, seed,
                                       _ptr(out), _ptr(fb), _stream_ptr(stream)))
        return out, fb

    # -- launch configuration of the batched form ----------------------------------
    def launch_config(self) -> dict:
        c = LaunchConfig()
        check(lib().hepem_get_launch_config(self.h, C.byref(c)))
        return c.as_dict()

    def set_launch_config(self, cfg: dict | None):
        if cfg is None:
            check(lib().hepem_set_launch_config(self.h, None))
            return
        c = LaunchConfig()
        for k in range(11):
            c.block[k] = cfg["block"][k]
            c.ctas_per_sm[k] = cfg["ctas_per_sm"][k]
        c.sort_energy_bins = cfg["sort_energy_bins"]
        check(lib().hepem_set_launch_config(self.h, C.byref(c)))

    def set_table_l2_window(self, enable: bool) -> int:
        """Sets or clears the L2 persisting window over the tables of the
        batched forms' stage kernels; returns the window's size in bytes."""
        w = C.c_int64(0)
        check(lib().hepem_set_table_l2_window(self.h, int(bool(enable)), C.byref(w)))
        return w.value

    def autotune(self, state_in: dict, uniforms, n_uniform: int, seed: int, apply=True, stream=None) -> dict:
        """Times the batched step on this batch under every launch candidate;
        returns the fastest configuration (and applies it if `apply`)."""
        n = len(state_in["ekin"])
        sin = make_state_struct(state_in)
        c = LaunchConfig()
        check(lib().hepem_autotune(self.h, n, C.byref(sin), _ptr(uniforms) if n_uniform else None, n_uniform, seed,
                                   int(apply), C.byref(c), _stream_ptr(stream)))
        return c.as_dict()

    def step_host(self, state_in: dict, state_out: dict, uniforms: np.ndarray, n_uniform: int, seed: int,
                  res: dict, stream=None, mixed=False):
        """hepem_step_host (or hepem_step_host_mixed): host buffers in and out."""
        n = len(state_in["ekin"])
        cnt = StepCounters()
        sin, sout, sres = make_state_struct(state_in), make_state_struct(state_out), make_out_struct(res)
        fn = lib().hepem_step_host_mixed if mixed else lib().hepem_step_host
        check(fn(self.h, n, C.byref(sin), C.byref(sout), _ptr(uniforms), n_uniform, seed, C.byref(sres),
                 C.byref(cnt), _stream_ptr(stream)))
        return cnt


class Server:
    """Serving form: continuous batching of event requests (hepem_server_*).

    Requests are host SoA track batches (numpy dicts of STATE_FIELDS); results
    are RequestResult dicts, and optionally the final track state."""

    def __init__(self, ctx: Context, memory_budget_bytes: int, max_steps: int = 1000, max_requests: int = 4096,
                 min_energy: float = 1.0e-3, mixed: bool = False):
        self.ctx = ctx
        cfg = ServerConfig(int(memory_budget_bytes), int(max_steps), int(max_requests), float(min_energy),
                           int(mixed), 0)
        h = _vp()
        check(lib().hepem_server_create(ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = {}

    @property
    def capacity(self) -> int:
        c = C.c_int64()
        check(lib().hepem_server_capacity(self.h, C.byref(c)))
        return c.value

    def submit(self, tracks: dict, seed: int) -> int:
        n = len(tracks["ekin"])
        arrs = {f: np.ascontiguousarray(tracks[f], dtype=dt) for f, dt in STATE_FIELDS}
        st = make_state_struct(arrs)
        rid = C.c_int64()
        check(lib().hepem_server_submit(self.h, n, C.byref(st), seed, C.byref(rid)))
        self._keep[rid.value] = n
        return rid.value

    def _final(self, rid, want_tracks):
        if not want_tracks:
            return None, None
        n = self._keep[rid]
        arrs = {f: np.zeros(n, dtype=dt) for f, dt in STATE_FIELDS}
        return arrs, make_state_struct(arrs)

    def poll(self, rid: int, want_tracks: bool = False):
        """None while running, else (result dict, final tracks or None)."""
        done = C.c_int32()
        res = RequestResult()
        arrs, st = self._final(rid, want_tracks)
        rc = lib().hepem_server_poll(self.h, rid, C.byref(done), C.byref(res), C.byref(st) if st else None)
        if rc not in (0, STATUS_CANCELLED):
            check(rc)
        if not done.value:
            return None
        self._keep.pop(rid, None)
        return res.as_dict(), arrs

    def wait(self, rid: int, timeout_s: float = 600.0, want_tracks: bool = False):
        res = RequestResult()
        arrs, st = self._final(rid, want_tracks)
        rc = lib().hepem_server_wait(self.h, rid, timeout_s, C.byref(res), C.byref(st) if st else None)
        if rc not in (0, STATUS_CANCELLED):
            check(rc)
        self._keep.pop(rid, None)
        return res.as_dict(), arrs

    def cancel(self, rid: int):
        check(lib().hepem_server_cancel(self.h, rid))

    def snapshot(self) -> bytes:
        """hepem_server_snapshot: the unfinished requests as of the last
        completed iteration (they keep running here)."""
        L = lib()
        while True:
            size = C.c_size_t()
            check(L.hepem_server_snapshot(self.h, None, 0, C.byref(size)))
            buf = C.create_string_buffer(size.value)
            got = C.c_size_t()
            rc = L.hepem_server_snapshot(self.h, buf, size.value, C.byref(got))
            if rc == 0:
                return buf.raw[:got.value]
            if got.value <= size.value:   # not a size change between the two calls
                check(rc)

    def resume(self, snap: bytes) -> dict:
        """hepem_server_resume: submits the snapshot's requests; returns
        {snapshot request id: request id on this server}."""
        n = snapshot_check(snap)[0]
        old = (C.c_int64 * max(n, 1))()
        new = (C.c_int64 * max(n, 1))()
        got = C.c_int64()
        check(lib().hepem_server_resume(self.h, snap, len(snap), n, old, new, C.byref(got)))
        ids = {}
        for k, rec in enumerate(snapshot_records(snap)):
            ids[old[k]] = new[k]
            self._keep[new[k]] = rec["n"]
        return ids

    def stats(self) -> dict:
        s = ServerStats()
        check(lib().hepem_server_get_stats(self.h, C.byref(s)))
        return s.as_dict()

    def reset_stats(self):
        check(lib().hepem_server_reset_stats(self.h))

    def close(self):
        if getattr(self, "h", None):
            lib().hepem_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def snapshot_check(snap: bytes):
    """Validates a server snapshot (no GPU needed); returns (requests, tracks)."""
    nr, nt = C.c_int64(), C.c_int64()
    check(lib().hepem_server_snapshot_check(snap, len(snap), C.byref(nr), C.byref(nt)))
    return nr.value, nt.value


def snapshot_records(snap: bytes) -> list:
    """The request records of a validated snapshot: id, n, seed, steps,
    admitted, cancelled, and the track state (numpy arrays of STATE_FIELDS)."""
    snapshot_check(snap)
    nreq = int(np.frombuffer(snap, dtype=np.uint64, count=1, offset=16)[0])
    off, out = 32, []
    for _ in range(nreq):
        rid, n = (int(x) for x in np.frombuffer(snap, dtype=np.int64, count=2, offset=off))
        seed = int(np.frombuffer(snap, dtype=np.uint64, count=1, offset=off + 16)[0])
        steps = int(np.frombuffer(snap, dtype=np.int32, count=1, offset=off + 24)[0])
        admitted, cancelled = snap[off + 28], snap[off + 29]
        off += 32
        state = {}
        for f, dt in STATE_FIELDS:
            a = np.frombuffer(snap, dtype=dt, count=n, offset=off)
            state[f] = a.copy()
            off += a.nbytes
        sums = {}
        for f, dt in (("edep", np.float64), ("e_secondaries", np.float64), ("n_secondaries", np.int32),
                      ("track_steps", np.int32)):
            a = np.frombuffer(snap, dtype=dt, count=n, offset=off)
            sums[f] = a.copy()
            off += a.nbytes
        out.append(dict(id=rid, n=n, seed=seed, steps=steps, admitted=bool(admitted), cancelled=bool(cancelled),
                        state=state, sums=sums))
    return out


def image_from_json(json_text) -> bytes:
    """Binary image of the table arena of a G4HepEmState JSON document (no GPU needed)."""
    if isinstance(json_text, str):
        json_text = json_text.encode()
    size = C.c_size_t()
    check(lib().hepem_image_from_json(json_text, len(json_text), None, 0, C.byref(size)))
    buf = C.create_string_buffer(size.value)
    check(lib().hepem_image_from_json(json_text, len(json_text), buf, size.value, C.byref(size)))
    return buf.raw[:size.value]


def image_check(image: bytes) -> int:
    """Validates an image; returns its arena size in bytes."""
    nb = C.c_int64()
    check(lib().hepem_image_check(image, len(image), C.byref(nb)))
    return nb.value


def philox_uniform(seed: int, tid: int, k: int) -> float:
    return lib().hepem_philox_uniform(seed, tid, k)


def fill_uniforms(ids, n_uniform: int, seed: int, out=None, stream=None):
    import torch
    n = ids.numel()
    if out is None:
        out = torch.empty(n * n_uniform, dtype=torch.float64, device=ids.device)
    check(lib().hepem_fill_uniforms(n, _ptr(ids), n_uniform, seed, _ptr(out), _stream_ptr(stream)))
    return out


# -- helpers for numpy <-> torch batches -----------------------------------------------------
def alloc_out_numpy(n: int) -> dict:
    return {f: np.zeros(n * k, dtype=dt) for f, dt, k in OUT_FIELDS}


def alloc_out_torch(n: int, device="cuda") -> dict:
    import torch
    tmap = {np.float64: torch.float64, np.int8: torch.int8, np.uint8: torch.uint8, np.int32: torch.int32}
    return {f: torch.zeros(n * k, dtype=tmap[dt], device=device) for f, dt, k in OUT_FIELDS}


def state_to_torch(state: dict, device="cuda") -> dict:
    import torch
    return {f: torch.from_numpy(np.ascontiguousarray(state[f])).to(device) for f, _ in STATE_FIELDS}


def to_numpy(d: dict) -> dict:
    return {k: v.cpu().numpy() for k, v in d.items()}


def empty_state_torch(n: int, device="cuda") -> dict:
    import torch
    tmap = {np.float64: torch.float64, np.int8: torch.int8, np.uint8: torch.uint8, np.int32: torch.int32}
    return {f: torch.empty(n, dtype=tmap[dt], device=device) for f, dt in STATE_FIELDS}
