"""What a maintainer adds to the reference's code/pipeline/engine_adapter.py to
mine in-process through libsgfim.so instead of starting an engine executable.

It needs nothing but ctypes and the built library: run_gb300(fimi_path,
min_count) returns the same {'ok', 'mfis': {frozenset(original ids): support}}
shape that the adapter's run_tensorfim returns, with mine_mfi's complete MFI
set (SGFIM_ROOTS_ALL).  The library path defaults to the in-tree build next to
this file; SGFIM_LIB overrides it.
"""
import ctypes as C
import os

LIB = os.environ.get("SGFIM_LIB", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                               "_lib", "libsgfim.so"))
_sg = C.CDLL(LIB)


class _Params(C.Structure):      # sgfim_mine_params
    _fields_ = [("min_count", C.c_uint32), ("root_rule", C.c_uint32), ("roots", C.POINTER(C.c_uint32)),
                ("n_roots", C.c_uint32), ("root_min_count", C.c_uint32), ("order", C.c_uint32),
                ("time_limit_s", C.c_double), ("node_limit", C.c_uint64), ("record_trace", C.c_uint32)]


class _Result(C.Structure):      # sgfim_result (leading fields; the rest is never touched here)
    _fields_ = [("n_sets", C.c_uint64), ("set_ptr", C.POINTER(C.c_uint64)),
                ("items", C.POINTER(C.c_uint32)), ("support", C.POINTER(C.c_uint32))]


_sg.sgfim_last_error.restype = C.c_char_p


def run_gb300(fimi_path, min_count):
    h = C.c_void_p()
    if _sg.sgfim_open(None, C.byref(h)) != 0:          # device 0, default budget
        return {"ok": False, "mfis": {}}
    try:
        if _sg.sgfim_load_fimi(h, fimi_path.encode()) != 0:
            return {"ok": False, "mfis": {}, "error": _sg.sgfim_last_error(h).decode()}
        p, res = _Params(min_count=max(1, int(min_count))), C.POINTER(_Result)()
        if _sg.sgfim_mine(h, C.byref(p), C.byref(res)) != 0:
            return {"ok": False, "mfis": {}, "error": _sg.sgfim_last_error(h).decode()}
        r = res.contents
        mfis = {frozenset(r.items[k] for k in range(r.set_ptr[i], r.set_ptr[i + 1])): r.support[i]
                for i in range(r.n_sets)}
        _sg.sgfim_result_free(res)
        return {"ok": True, "mfis": mfis}
    finally:
        _sg.sgfim_close(h)
