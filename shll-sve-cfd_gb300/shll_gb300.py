"""ctypes binding of libshll_gb300.so (the C-ABI declared in include/shll.h).

This is the host-side mirror of the reference's solver stages (archembaud/shll-sve-cfd,
base-c/base_shll.c:28-225): a Context owns one problem on the GPU and exposes
init_state (Allocate_and_Init_Memory + Compute_U_from_P + Compute_P_from_U), the four stages,
run (the time loop), and the results.  There is no CPU fallback: loading fails loudly if the
library has not been built.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libshll_gb300.so")

OK, ERR_ARG, ERR_CUDA, ERR_STATE, ERR_NOMEM, ERR_NUMERIC, ERR_TIMEOUT, ERR_UNSUPPORTED = 0, -1, -2, -3, -4, -5, -6, -7
PREC_F64, PREC_F64_EXACT, PREC_F32_EXACT, PREC_MIXED_F64, PREC_MIXED_KAHAN = 0, 1, 2, 3, 4
IC_SOD, IC_REF_BOX2D, IC_CIRCLE2D, IC_FOUR_SHOCK2D, IC_USER, IC_QUADRANTS2D = 0, 1, 2, 3, 4, 5
PRECISIONS = {"f64": PREC_F64, "f64_exact": PREC_F64_EXACT, "f32_exact": PREC_F32_EXACT,
              "mixed_f64": PREC_MIXED_F64, "mixed_kahan": PREC_MIXED_KAHAN}


class Ic(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("x_d", ctypes.c_double),
                ("rho_l", ctypes.c_double), ("u_l", ctypes.c_double), ("T_l", ctypes.c_double),
                ("rho_r", ctypes.c_double), ("u_r", ctypes.c_double), ("T_r", ctypes.c_double),
                ("cx", ctypes.c_double), ("cy", ctypes.c_double), ("radius", ctypes.c_double)]


class Params(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("order", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("gamma", ctypes.c_double), ("R", ctypes.c_double), ("cfl", ctypes.c_double),
                ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("t_end", ctypes.c_double),
                ("n_steps", ctypes.c_long), ("precision", ctypes.c_int), ("limiter", ctypes.c_int),
                ("mc_alpha", ctypes.c_double), ("fold_steps", ctypes.c_int), ("clock_f32", ctypes.c_int),
                ("ic", Ic)]


class ShllError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None

EXPORTS = [
    "shll_params_default", "shll_steps_for", "shll_create", "shll_destroy", "shll_last_error",
    "shll_status_string", "shll_set_stream", "shll_init_state", "shll_set_primitives",
    "shll_compute_U_from_P", "shll_compute_P_from_U", "shll_compute_F_from_P", "shll_update_U_from_F",
    "shll_step", "shll_run", "shll_steps_taken", "shll_get_primitives", "shll_get_conserved",
    "shll_get_fluxes", "shll_totals", "shll_save_results", "shll_batch_create", "shll_batch_run",
    "shll_batch_get_primitives", "shll_batch_totals", "shll_batch_cell_updates", "shll_batch_last_error",
    "shll_batch_destroy", "shll_ref_configure", "shll_ref_context", "Allocate_and_Init_Memory",
    "Compute_U_from_P", "Compute_P_from_U", "Compute_F_from_P", "Update_U_from_F", "Save_Results",
    "Free_Memory", "shll_ref_dt", "shll_checkpoint", "shll_restore", "shll_kernel_launches",
    "shll_batch_set_stream", "shll_batch_item_status", "shll_set_graph_replay", "shll_batch_checkpoint",
    "shll_batch_restore", "shll_batch_autotune", "shll_batch_tuning", "shll_autotune", "shll_tuning",
    "shll_set_resident", "shll_debug_stall_chunk", "shll_batch_set_primitives", "shll_initial_primitives",
    "shll_batch_set_all_primitives", "shll_batch_get_all_primitives", "shll_set_pair_flux",
    "shll_set_cluster_runs",
]


def lib():
    """Loads the library (built by build.py / __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libshll_gb300.so not built ({LIB_PATH}); run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        vp = ctypes.c_void_p
        P = ctypes.POINTER(Params)
        L.shll_params_default.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.shll_params_default.restype = None
        L.shll_steps_for.argtypes = [P]
        L.shll_steps_for.restype = ctypes.c_long
        L.shll_create.argtypes = [P, ctypes.POINTER(vp)]
        L.shll_destroy.argtypes = [vp]
        L.shll_destroy.restype = None
        L.shll_last_error.argtypes = [vp]
        L.shll_last_error.restype = ctypes.c_char_p
        L.shll_status_string.argtypes = [ctypes.c_int]
        L.shll_status_string.restype = ctypes.c_char_p
        L.shll_set_stream.argtypes = [vp, vp]
        for f in ("shll_init_state", "shll_compute_U_from_P", "shll_compute_P_from_U", "shll_compute_F_from_P",
                  "shll_update_U_from_F"):
            getattr(L, f).argtypes = [vp]
        L.shll_set_primitives.argtypes = [vp, dp, dp, dp, dp]
        L.shll_step.argtypes = [vp, ctypes.c_long]
        L.shll_run.argtypes = [vp, ctypes.POINTER(ctypes.c_long)]
        L.shll_steps_taken.argtypes = [vp]
        L.shll_steps_taken.restype = ctypes.c_long
        L.shll_get_primitives.argtypes = [vp, dp, dp, dp, dp]
        L.shll_get_conserved.argtypes = [vp, dp]
        L.shll_get_fluxes.argtypes = [vp, dp, dp, dp, dp]
        L.shll_totals.argtypes = [vp, dp]
        L.shll_save_results.argtypes = [vp, ctypes.c_char_p]
        L.shll_batch_create.argtypes = [P, ctypes.c_int, ctypes.POINTER(vp)]
        L.shll_batch_run.argtypes = [vp]
        L.shll_batch_set_stream.argtypes = [vp, vp]
        L.shll_batch_item_status.argtypes = [vp, ctypes.c_int]
        L.shll_batch_get_primitives.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp]
        L.shll_batch_set_primitives.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp]
        L.shll_initial_primitives.argtypes = [P, dp, dp, dp, dp]
        L.shll_batch_set_all_primitives.argtypes = [vp, dp]
        L.shll_batch_get_all_primitives.argtypes = [vp, dp]
        L.shll_batch_totals.argtypes = [vp, ctypes.c_int, dp]
        L.shll_batch_cell_updates.argtypes = [vp]
        L.shll_batch_cell_updates.restype = ctypes.c_long
        L.shll_batch_last_error.argtypes = [vp]
        L.shll_batch_last_error.restype = ctypes.c_char_p
        L.shll_batch_destroy.argtypes = [vp]
        L.shll_batch_destroy.restype = None
        L.shll_ref_configure.argtypes = [P]
        L.shll_ref_context.restype = vp
        L.shll_ref_dt.restype = ctypes.c_double
        L.shll_checkpoint.argtypes = [vp]
        L.shll_restore.argtypes = [vp]
        L.shll_kernel_launches.restype = ctypes.c_long
        for f in ("Allocate_and_Init_Memory", "Compute_U_from_P", "Compute_P_from_U", "Compute_F_from_P",
                  "Update_U_from_F", "Save_Results", "Free_Memory"):
            getattr(L, f).restype = None
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def params(dim=1, order=1, nx=256, ny=None, precision="f64", **kw):
    """Reference defaults for (dim, order) with overrides; ic_* keys set the initial data."""
    p = Params()
    lib().shll_params_default(ctypes.byref(p), dim, order)
    p.nx = nx
    p.ny = (ny if ny is not None else nx) if dim == 2 else 1
    p.precision = PRECISIONS[precision] if isinstance(precision, str) else precision
    for k, v in kw.items():
        if k.startswith("ic_"):
            setattr(p.ic, k[3:], v)
        else:
            setattr(p, k, v)
    return p


def steps_for(p):
    return lib().shll_steps_for(ctypes.byref(p))


def initial_primitives(p, out=None):
    """(nv, n) array: the initial rho, u, [v,] T of p's descriptor (what init_state loads), into
    `out` (C-contiguous float64 of that shape) when given."""
    nv = 4 if p.dim == 2 else 3
    n = p.nx * (p.ny if p.dim == 2 else 1)
    if out is None:
        out = np.zeros((nv, n))
    assert out.shape == (nv, n) and out.dtype == np.float64 and out.flags.c_contiguous
    rc = lib().shll_initial_primitives(ctypes.byref(p), _dp(out[0]), _dp(out[1]), _dp(out[2]) if nv == 4 else None,
                                       _dp(out[nv - 1]))
    if rc != OK:
        raise ShllError(rc, "initial_primitives: invalid parameters")
    return out


def kernel_launches():
    return lib().shll_kernel_launches()


def set_graph_replay(on):
    """Replay captured launch sequences of repeated mixed-precision 1D runs (default on)."""
    lib().shll_set_graph_replay(1 if on else 0)


def set_resident(on):
    """Run single-wave mixed-precision 1D runs as one resident launch (default on)."""
    lib().shll_set_resident(1 if on else 0)


def set_pair_flux(on):
    """Evaluate first-order fluxes in double-FP32 arithmetic where the flow is supersonic (default 1; 0 off,
    2 in every first-order chunk)."""
    lib().shll_set_pair_flux(int(on))


def set_cluster_runs(on):
    """Run 1D tubes of 2..16 chunks as one thread-block cluster each (default off)."""
    lib().shll_set_cluster_runs(1 if on else 0)


def debug_stall_chunk(chunk):
    """Test hook: in resident runs, chunk `chunk` never publishes its progress (-1: off)."""
    lib().shll_debug_stall_chunk(int(chunk))


class Context:
    """One problem on the GPU (a shll_ctx)."""

    def __init__(self, p):
        self.p = p
        self.h = ctypes.c_void_p()
        rc = lib().shll_create(ctypes.byref(p), ctypes.byref(self.h))
        if rc != OK:
            raise ShllError(rc, "shll_create failed: " + lib().shll_status_string(rc).decode())
        self.n = p.nx * (p.ny if p.dim == 2 else 1)
        self.nv = 4 if p.dim == 2 else 3

    def _ck(self, rc, what):
        if rc != OK:
            raise ShllError(rc, f"{what}: {lib().shll_last_error(self.h).decode()}")
        return rc

    def close(self):
        if self.h:
            lib().shll_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_state(self):
        return self._ck(lib().shll_init_state(self.h), "init_state")

    def set_primitives(self, rho, u, T, v=None):
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (rho, u, T)]
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        return self._ck(lib().shll_set_primitives(self.h, _dp(arrs[0]), _dp(arrs[1]), _dp(vv), _dp(arrs[2])),
                        "set_primitives")

    def compute_U_from_P(self):
        return self._ck(lib().shll_compute_U_from_P(self.h), "Compute_U_from_P")

    def compute_P_from_U(self):
        return self._ck(lib().shll_compute_P_from_U(self.h), "Compute_P_from_U")

    def compute_F_from_P(self):
        return self._ck(lib().shll_compute_F_from_P(self.h), "Compute_F_from_P")

    def update_U_from_F(self):
        return self._ck(lib().shll_update_U_from_F(self.h), "Update_U_from_F")

    def step(self, n):
        return self._ck(lib().shll_step(self.h, n), "step")

    def run(self):
        s = ctypes.c_long()
        self._ck(lib().shll_run(self.h, ctypes.byref(s)), "run")
        return s.value

    @property
    def steps_taken(self):
        return lib().shll_steps_taken(self.h)

    def primitives(self, out=None):
        """(nv, n) array: rho, u, [v,] T (into `out`, a C-contiguous float64 array of that shape,
        for instance a view of pinned host memory, when given)."""
        if out is None:
            out = np.zeros((self.nv, self.n))
        assert out.shape == (self.nv, self.n) and out.dtype == np.float64 and out.flags.c_contiguous
        if self.nv == 3:
            self._ck(lib().shll_get_primitives(self.h, _dp(out[0]), _dp(out[1]), None, _dp(out[2])), "primitives")
        else:
            self._ck(lib().shll_get_primitives(self.h, _dp(out[0]), _dp(out[1]), _dp(out[2]), _dp(out[3])),
                     "primitives")
        return out

    def conserved(self):
        out = np.zeros((self.nv, self.n))
        self._ck(lib().shll_get_conserved(self.h, _dp(out)), "conserved")
        return out

    def fluxes(self):
        fp, fm = np.zeros((self.nv, self.n)), np.zeros((self.nv, self.n))
        if self.nv == 4:
            hp, hm = np.zeros((self.nv, self.n)), np.zeros((self.nv, self.n))
            self._ck(lib().shll_get_fluxes(self.h, _dp(fp), _dp(fm), _dp(hp), _dp(hm)), "fluxes")
            return fp, fm, hp, hm
        self._ck(lib().shll_get_fluxes(self.h, _dp(fp), _dp(fm), None, None), "fluxes")
        return fp, fm

    def totals(self):
        out = np.zeros(self.nv)
        self._ck(lib().shll_totals(self.h, _dp(out)), "totals")
        return out

    def autotune(self, trial_steps=0):
        """Picks the 1D sweep length and fold window, or the 2D fold window, by timed trials (state restored)."""
        return self._ck(lib().shll_autotune(self.h, trial_steps), "autotune")

    def tuning(self):
        b, f, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._ck(lib().shll_tuning(self.h, ctypes.byref(b), ctypes.byref(f), ctypes.byref(c)), "tuning")
        return b.value, f.value, c.value

    def checkpoint(self):
        return self._ck(lib().shll_checkpoint(self.h), "checkpoint")

    def restore(self):
        return self._ck(lib().shll_restore(self.h), "restore")

    def set_stream(self, stream_ptr):
        return self._ck(lib().shll_set_stream(self.h, stream_ptr), "set_stream")

    def save_results(self, path):
        return self._ck(lib().shll_save_results(self.h, path.encode()), "save_results")


class Batch:
    """Many independent tubes or domains advanced together (a shll_batch)."""

    def __init__(self, items):
        arr = (Params * len(items))(*items)
        self.items = items
        self.h = ctypes.c_void_p()
        rc = lib().shll_batch_create(arr, len(items), ctypes.byref(self.h))
        if rc != OK:
            raise ShllError(rc, "shll_batch_create failed: " + lib().shll_status_string(rc).decode())

    def _ck(self, rc, what):
        if rc != OK:
            raise ShllError(rc, f"{what}: {lib().shll_batch_last_error(self.h).decode()}")

    def run(self, allow_numeric=False):
        """Runs every item to its end.  allow_numeric: do not raise when some items reached a
        non-positive/NaN state (check item_status)."""
        rc = lib().shll_batch_run(self.h)
        if rc == ERR_NUMERIC and allow_numeric:
            return rc
        self._ck(rc, "batch_run")
        return rc

    def autotune(self, trial_steps=0):
        """Picks sweep length and fold window per size class by timed trials (state restored)."""
        return self._ck(lib().shll_batch_autotune(self.h, trial_steps), "batch_autotune")

    def tuning(self, i):
        """(sweep length, fold interval) in steps and owned cells per chunk chosen for item i."""
        b, f, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._ck(lib().shll_batch_tuning(self.h, i, ctypes.byref(b), ctypes.byref(f), ctypes.byref(c)), "batch_tuning")
        return b.value, f.value, c.value

    def checkpoint(self):
        """Device-side copy of the state (mixed-precision 1D batches)."""
        return self._ck(lib().shll_batch_checkpoint(self.h), "batch_checkpoint")

    def restore(self):
        """Back to the last checkpoint (also clears breakdown flags raised since)."""
        return self._ck(lib().shll_batch_restore(self.h), "batch_restore")

    def item_status(self, i):
        return lib().shll_batch_item_status(self.h, i)

    def set_stream(self, stream_ptr):
        self._ck(lib().shll_batch_set_stream(self.h, stream_ptr), "batch_set_stream")

    def set_primitives(self, i, rho, u, T, v=None):
        """Replaces item i's state (host arrays, copied as given and converted on the device)."""
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (rho, u, T)]
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        return self._ck(lib().shll_batch_set_primitives(self.h, i, _dp(arrs[0]), _dp(arrs[1]), _dp(vv), _dp(arrs[2])),
                        "batch_set_primitives")

    def packed_size(self):
        """Doubles of the packed layout: item after item, each item's planes rho, u, [v,] T."""
        return sum((4 if p.dim == 2 else 3) * p.nx * (p.ny if p.dim == 2 else 1) for p in self.items)

    def set_all_primitives(self, packed):
        """Every item's state from one packed host array (see packed_size)."""
        assert packed.dtype == np.float64 and packed.flags.c_contiguous and packed.size == self.packed_size()
        return self._ck(lib().shll_batch_set_all_primitives(self.h, _dp(packed)), "batch_set_all_primitives")

    def get_all_primitives(self, out=None):
        """Every item's primitives into one packed array (see packed_size)."""
        if out is None:
            out = np.zeros(self.packed_size())
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.packed_size()
        self._ck(lib().shll_batch_get_all_primitives(self.h, _dp(out)), "batch_get_all_primitives")
        return out

    def primitives(self, i, out=None):
        """(nv, n) array of item i: rho, u, [v,] T (into `out` when given, as Context.primitives)."""
        p = self.items[i]
        n = p.nx * (p.ny if p.dim == 2 else 1)
        nv = 4 if p.dim == 2 else 3
        if out is None:
            out = np.zeros((nv, n))
        assert out.shape == (nv, n) and out.dtype == np.float64 and out.flags.c_contiguous
        if nv == 3:
            self._ck(lib().shll_batch_get_primitives(self.h, i, _dp(out[0]), _dp(out[1]), None, _dp(out[2])), "prims")
        else:
            self._ck(lib().shll_batch_get_primitives(self.h, i, _dp(out[0]), _dp(out[1]), _dp(out[2]), _dp(out[3])),
                     "prims")
        return out

    def totals(self, i):
        nv = 4 if self.items[i].dim == 2 else 3
        out = np.zeros(nv)
        self._ck(lib().shll_batch_totals(self.h, i, _dp(out)), "totals")
        return out

    @property
    def cell_updates(self):
        return lib().shll_batch_cell_updates(self.h)

    def close(self):
        if self.h:
            lib().shll_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
