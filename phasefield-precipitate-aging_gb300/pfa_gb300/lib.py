"""ctypes binding of libpfa_gb300.so (the extern "C" surface of include/pfa_gb300.h).

``Grid2D`` follows the reference's call sequence (src/main.cpp:229-321):
init_cuda with the host fields, a step loop of device_evolution + pointer
swap (optionally with nucleation), read_out_result.  The library is loaded
from this package directory; if it is missing, import fails loudly -- there
is no CPU fallback.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libpfa_gb300.so")

FP64, FP32, FP32_KPHI = 0, 1, 2
MOBILITY_CONSTANT, MOBILITY_VARIABLE = 0, 1
MODE_FUSED, MODE_COMPAT = 0, 1
NUC_REFERENCE_GEOMETRY, NUC_FIXED_GEOMETRY = 0, 1
PRECISIONS = {"fp64": FP64, "fp32": FP32, "fp32k": FP32_KPHI}

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i, _d = ctypes.c_int, ctypes.c_double


class CudaData(ctypes.Structure):
    """Layout of struct CudaData, src/type.h:58-107."""
    _fields_ = ([("prng", ctypes.c_void_p)] +
                [(n, ctypes.c_void_p) for n in ("str_A", "str_B", "str_C", "str_D")] +
                [(n, ctypes.c_void_p) for n in ("ev_A", "ev_B", "ev_C", "ev_D")] +
                [(n, _dp) for n in ("conc_Ni", "phi", "conc_Cr_old", "conc_Cr_new",
                                    "conc_Nb_old", "conc_Nb_new", "phi_del_old", "phi_del_new",
                                    "phi_lav_old", "phi_lav_new", "conc_Cr_gam", "conc_Cr_del",
                                    "conc_Cr_lav", "conc_Nb_gam", "conc_Nb_del", "conc_Nb_lav")])


IC_MAX_BANDS, IC_MAX_PARTICLES = 16, 64


class IcRecipe(ctypes.Structure):
    """Layout of pfa_ic_recipe (pfa_gb300.h): a grid the device builds."""
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i),
                ("matrix", _d * 2), ("enrich", _d * 2), ("noise", _d), ("seed", ctypes.c_uint64),
                ("n_bands", _i), ("band", (_i * 2) * IC_MAX_BANDS),
                ("n_particles", _i), ("centre", (_d * 3) * IC_MAX_PARTICLES),
                ("radius", _d * IC_MAX_PARTICLES), ("phase", _i * IC_MAX_PARTICLES),
                ("dx", _d), ("width", _d), ("profile", _i), ("bell_sigma", _d * 2),
                ("bell_range", _d * 2), ("bell_x0", _d), ("particle_mode", _i)]


def ic_recipe(rec):
    """IcRecipe from a recipe dict: nx, ny, nz (interior; nz <= 1 for 2D),
    matrix, enrich, noise, seed, bands [(lo, hi)], particles
    [(x, y, z, radius, phase)], dx, width."""
    r = IcRecipe()
    r.nx, r.ny, r.nz = int(rec["nx"]), int(rec["ny"]), int(rec.get("nz", 0))
    r.matrix[:] = rec["matrix"]
    r.enrich[:] = rec["enrich"]
    r.noise = rec["noise"]
    r.seed = int(rec["seed"])
    bands, parts = rec.get("bands", []), rec.get("particles", [])
    if len(bands) > IC_MAX_BANDS or len(parts) > IC_MAX_PARTICLES:
        raise ValueError("recipe: too many bands or particles")
    r.n_bands = len(bands)
    for k, (lo, hi) in enumerate(bands):
        r.band[k][0], r.band[k][1] = int(lo), int(hi)
    r.n_particles = len(parts)
    for k, (x, y, z, rad, ph) in enumerate(parts):
        r.centre[k][0], r.centre[k][1], r.centre[k][2] = x, y, z
        r.radius[k] = rad
        r.phase[k] = int(ph)
    r.dx, r.width = rec["dx"], rec["width"]
    r.profile = int(rec.get("profile", 0))
    r.bell_sigma[:] = rec.get("bell_sigma", (0.0, 0.0))
    r.bell_range[:] = rec.get("bell_range", (0.0, 0.0))
    r.bell_x0 = rec.get("bell_x0", 0.0)
    r.particle_mode = int(rec.get("particle_mode", 0))
    return r


def ic_shape(rec):
    """Shape of the recipe's fields with the ghost ring."""
    if int(rec.get("nz", 0)) > 1:
        return (rec["nz"] + 2, rec["ny"] + 2, rec["nx"] + 2)
    return (rec["ny"] + 2, rec["nx"] + 2)


def ic_generate(rec, ptrs, stream=None):
    """Build the recipe's four fields in caller-owned device arrays (device
    addresses, reference layout) on `stream` (a cudaStream_t value or None)."""
    r = ic_recipe(rec)
    check(load().pfa_ic_generate(ctypes.byref(r), *[ctypes.c_void_p(int(q)) for q in ptrs],
                                 ctypes.c_void_p(stream or 0)), "pfa_ic_generate")


_lib = None


def load():
    """Load (and type) the library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with pfa_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER(CudaData)
    sig = {
        "pfa_last_error": (_i, []),
        "pfa_error_string": (ctypes.c_char_p, [_i]),
        "pfa_last_error_message": (ctypes.c_char_p, []),
        "pfa_clear_error": (None, []),
        "pfa_set_device": (_i, [_i]),
        "pfa_device_count": (_i, []),
        "pfa_set_mode": (_i, [P, _i]),
        "pfa_set_precision": (_i, [P, _i]),
        "pfa_set_nucleation": (_i, [P, ctypes.c_uint64, _i]),
        "pfa_set_mobility": (_i, [P, _i]),
        "pfa_get_counters": (_i, [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
        "pfa_set_counters": (_i, [P, ctypes.c_uint64, ctypes.c_uint64]),
        "pfa_f32_state_bytes": (ctypes.c_size_t, [P]),
        "pfa_read_f32_state": (_i, [P, ctypes.c_void_p, ctypes.c_size_t]),
        "pfa_write_f32_state": (_i, [P, ctypes.c_void_p, ctypes.c_size_t]),
        "pfa_device_mobilities": (_i, [P, _i, _i, _i, _i, _i]),
        "pfa_mobility_boundaries": (_i, [P, _i, _i, _i, _i, _i]),
        "pfa_set_nucleation_args": (_i, [P, _i, _d, _d, _d, _d, _d, _d, _d]),
        "pfa_init_cuda": (_i, [P, _i, _i, _i, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
        "pfa_free_cuda": (_i, [P]),
        "pfa_read_out_result": (_i, [P, _dp, _dp, _dp, _dp, _i, _i]),
        "pfa_upload_fields": (_i, [P, _dp, _dp, _dp, _dp, _i, _i]),
        "pfa_read_out_result_async": (_i, [P, _dp, _dp, _dp, _dp, _i, _i]),
        "pfa_upload_fields_async": (_i, [P, _dp, _dp, _dp, _dp, _i, _i]),
        "pfa_device_boundaries": (_i, [P, _i, _i, _i, _i, _i]),
        "pfa_device_fictitious": (_i, [P, _i, _i, _i, _i, _i]),
        "pfa_fictitious_boundaries": (_i, [P, _i, _i, _i, _i, _i]),
        "pfa_device_laplacian": (_i, [P, _i, _i, _i, _i, _i, _d, _d]),
        "pfa_device_laplacian_boundaries": (_i, [P, _i, _i, _i, _i, _i]),
        "pfa_device_evolution": (_i, [P, _i, _i, _i, _i, _i, _d, _d]),
        "pfa_device_init_prng": (_i, [P, _i, _i, _i, _i, _i]),
        "pfa_device_nucleation": (_i, [P, _i, _i, _i, _i, _i] + [_d] * 8),
        "pfa_device_dataviz": (_i, [P, _dp, _dp, _dp, _dp, _dp, _dp, _i, _i]),
        "pfa_swap": (_i, [P]),
        "pfa_run": (_i, [P, _i, _d, _d]),
        "pfa_run_timed": (_i, [P, _i, _d, _d, _fp]),
        "pfa_sync": (_i, [P]),
        "pfa_stream": (ctypes.c_void_p, [P]),
        "pfa_last_nucleation_events": (_i, [P, ctypes.POINTER(ctypes.c_int64),
                                            ctypes.POINTER(ctypes.c_int32), _i]),
        "pfa_summarize": (_i, [P, _dp]),
        "pfa_model_params": (_i, [_d, _d, _d, _d, _d, _i, _i, _dp]),
        "pfa_model_fast_coef": (_i, [_fp, _i]),
        "pfa_philox_block": (_i, [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint64,
                                  ctypes.POINTER(ctypes.c_uint32), _i]),
        "pfa_summarize_fields_noalloc": (_i, [ctypes.c_void_p] * 4 + [_i, _i, ctypes.c_void_p,
                                                                      ctypes.c_void_p]),
        "pfa3d_create": (_i, [ctypes.POINTER(ctypes.c_void_p), _i, _i, _i, _dp, _dp, _dp, _dp,
                              _dp, _dp, _i]),
        "pfa3d_run": (_i, [ctypes.c_void_p, _i]),
        "pfa3d_get_counters": (_i, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                    ctypes.POINTER(ctypes.c_uint64)]),
        "pfa3d_set_counters": (_i, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64]),
        "pfa3d_f32_state_bytes": (ctypes.c_size_t, [ctypes.c_void_p]),
        "pfa3d_read_f32_state": (_i, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
        "pfa3d_write_f32_state": (_i, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
        "pfa3d_run_timed": (_i, [ctypes.c_void_p, _i, _fp]),
        "pfa3d_read": (_i, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
        "pfa3d_upload": (_i, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
        "pfa3d_read_async": (_i, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
        "pfa3d_upload_async": (_i, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
        "pfa3d_summarize": (_i, [ctypes.c_void_p, _dp]),
        "pfa3d_destroy": (_i, [ctypes.c_void_p]),
        "pfa3d_test_skip_plane": (_i, [ctypes.c_void_p, _i]),
        "pfa3d_footprint": (ctypes.c_size_t, [_i, _i, _i, _i]),
        "pfa3d_sync": (_i, [ctypes.c_void_p]),
        "pfa3d_summarize_energy": (_i, [ctypes.c_void_p, _d, _dp]),
        "pfa3d_set_nucleation": (_i, [ctypes.c_void_p, ctypes.c_uint64, _i] + [_d] * 7),
        "pfa3d_last_nucleation_events": (_i, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                              ctypes.POINTER(ctypes.c_int32), _i]),
        "pfa_summarize_energy": (_i, [P, _d, _d, _d, _dp, _dp, _dp]),
        "pfa_batch_footprint": (ctypes.c_size_t, [_i, _i]),
        "pfa_batch_create": (_i, [ctypes.POINTER(ctypes.c_void_p), _dp, _dp, ctypes.c_size_t]),
        "pfa_batch_add": (_i, [ctypes.c_void_p, _i, _i, _dp, _dp, _dp, _dp,
                               ctypes.POINTER(_i)]),
        "pfa_batch_remove": (_i, [ctypes.c_void_p, _i]),
        "pfa_batch_read": (_i, [ctypes.c_void_p, _i, _dp, _dp, _dp, _dp]),
        "pfa_batch_read_async": (_i, [ctypes.c_void_p, _i, _dp, _dp, _dp, _dp]),
        "pfa_batch_run": (_i, [ctypes.c_void_p, _i]),
        "pfa_batch_run_timed": (_i, [ctypes.c_void_p, _i, _fp]),
        "pfa_batch_sync": (_i, [ctypes.c_void_p]),
        "pfa_batch_summarize": (_i, [ctypes.c_void_p, _i, _dp]),
        "pfa_batch_tune": (_i, [ctypes.c_void_p, _i, _fp]),
        "pfa_batch_set_launch": (_i, [ctypes.c_void_p, _i, _i, _i]),
        "pfa_batch_get_launch": (_i, [ctypes.c_void_p] + [ctypes.POINTER(_i)] * 4),
        "pfa_batch_info": (_i, [ctypes.c_void_p, ctypes.POINTER(_i),
                                ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
        "pfa_batch_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
        "pfa_batch_destroy": (_i, [ctypes.c_void_p]),
        "pfa_ic_generate": (_i, [ctypes.POINTER(IcRecipe)] + [ctypes.c_void_p] * 5),
        "pfa_split_block": (_i, [_dp, _fp, _fp, _i]),
        "pfa_batch_add_ic": (_i, [ctypes.c_void_p, ctypes.POINTER(IcRecipe), ctypes.POINTER(_i)]),
        "pfa3d_create_ic": (_i, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(IcRecipe), _dp,
                                 _dp, _i]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class PfaError(RuntimeError):
    pass


def check(rc, what=""):
    if rc != 0:
        L = load()
        msg = L.pfa_last_error_message().decode(errors="replace")
        raise PfaError(f"{what}: {L.pfa_error_string(rc).decode()} ({msg})")
    return rc


def _ptr(a):
    return a.ctypes.data_as(_dp)


def five_point_mask(dx, dy):
    """3x3 mask of five_point_Laplacian_stencil, src/mesh.cpp:187-196 (same
    floating-point expressions)."""
    m = np.zeros((3, 3))
    m[0, 1] = 1. / (dy * dy)
    m[1, 0] = 1. / (dx * dx)
    m[1, 1] = -2. * (dx * dx + dy * dy) / (dx * dx * dy * dy)
    m[1, 2] = 1. / (dx * dx)
    m[2, 1] = 1. / (dy * dy)
    return m


def nine_point_mask(dx, dy):
    """nine_point_Laplacian_stencil, src/mesh.cpp:198-213."""
    m = np.zeros((3, 3))
    m[0, 0] = 1. / (6. * dx * dy)
    m[0, 1] = 4. / (6. * dy * dy)
    m[0, 2] = 1. / (6. * dx * dy)
    m[1, 0] = 4. / (6. * dx * dx)
    m[1, 1] = -10. * (dx * dx + dy * dy) / (6. * dx * dx * dy * dy)
    m[1, 2] = 4. / (6. * dx * dx)
    m[2, 0] = 1. / (6. * dx * dy)
    m[2, 1] = 4. / (6. * dy * dy)
    m[2, 2] = 1. / (6. * dx * dy)
    return m


# checkpoint files: one .npz with the FP64 fields (cr, nb, pd, pl), the mask
# (2D), a JSON `meta` record and, for the FP32 forms, the raw records
CHECKPOINT_FORMAT = "pfa-gb300-checkpoint-1"


def _load_checkpoint(path, dim):
    """(meta, fields, mask or None, FP32 record bytes or None) of a checkpoint
    file written by Grid2D / Grid3D .checkpoint for a grid of `dim`
    dimensions; ValueError for anything else."""
    import json
    with np.load(path) as z:
        if "meta" not in z.files:
            raise ValueError(f"{path}: not a checkpoint file (no meta record)")
        meta = json.loads(str(z["meta"]))
        if meta.get("format") != CHECKPOINT_FORMAT:
            raise ValueError(f"{path}: checkpoint format {meta.get('format')!r}, "
                             f"expected {CHECKPOINT_FORMAT!r}")
        if meta.get("dim") != dim:
            raise ValueError(f"{path}: a {meta.get('dim')}D checkpoint, not {dim}D")
        fields = [z[k] for k in ("cr", "nb", "pd", "pl")]
        shape = fields[0].shape
        if len(shape) != dim or any(f.shape != shape for f in fields):
            raise ValueError(f"{path}: field arrays of shapes {[f.shape for f in fields]}")
        mask = z["mask"] if "mask" in z.files else None
        raw = np.ascontiguousarray(z["f32_state"]) if "f32_state" in z.files else None
    return meta, fields, mask, raw


def model_params(dx=5e-9, ifce_width=10e-9, xcr0=0.30, xnb0=0.02, meshres=None, dim=2,
                 dt_rule=1):
    """Model parameters from the library (src/main.cpp:252-268; see pfa_gb300.h)."""
    out = np.zeros(13)
    check(load().pfa_model_params(dx, ifce_width, xcr0, xnb0, dx if meshres is None else meshres,
                                  dim, dt_rule, _ptr(out)), "pfa_model_params")
    return {"D_Cr": [out[0], out[1]], "D_Nb": [out[2], out[3]], "kappa": [out[4], out[5]],
            "omega": [out[6], out[7]], "Lmob": [out[8], out[9]], "alpha": out[10],
            "dt": out[11], "rho": out[12], "dx": dx, "dy": dx, "dz": dx}


class Grid2D:
    """One 2D grid behind the reference's CudaData interface."""

    def __init__(self, fields, params, precision="fp64", mode="fused", mask=None,
                 mobility="constant"):
        L = load()
        self.L = L
        f = [np.ascontiguousarray(a, dtype=np.float64) for a in fields]
        self.ny, self.nx = f[0].shape
        self.params = dict(params)
        self.dev = CudaData()
        if mask is None:
            mask = five_point_mask(params["dx"], params.get("dy", params["dx"]))
        self.mask = np.ascontiguousarray(mask, dtype=np.float64)
        arr = lambda v: np.ascontiguousarray(v, dtype=np.float64)
        self._consts = [arr(params["kappa"]), arr(params["omega"]), arr(params["Lmob"]),
                        arr(params["D_Cr"]), arr(params["D_Nb"])]
        check(L.pfa_init_cuda(ctypes.byref(self.dev), self.nx, self.ny, 3, _ptr(self.mask),
                              *[_ptr(c) for c in self._consts], *[_ptr(a) for a in f]),
              "pfa_init_cuda")
        self._live = True
        self.mode, self.mobility, self.nucleation = mode, mobility, None
        if mode == "compat":
            check(L.pfa_set_mode(ctypes.byref(self.dev), MODE_COMPAT), "pfa_set_mode")
        self.set_precision(precision)
        if mobility != "constant":
            check(L.pfa_set_mobility(ctypes.byref(self.dev),
                                     {"variable": MOBILITY_VARIABLE}[mobility]), "pfa_set_mobility")

    @property
    def ref(self):
        return ctypes.byref(self.dev)

    def set_precision(self, precision):
        check(self.L.pfa_set_precision(self.ref, PRECISIONS[precision]), "pfa_set_precision")
        self.precision = precision

    def set_nucleation(self, seed=42, geometry=NUC_REFERENCE_GEOMETRY, interval=0,
                       sigma=(0.13, 0.13), unit_a=0.352e-9, d=None, dt_nuc=None):
        check(self.L.pfa_set_nucleation(self.ref, seed, geometry), "pfa_set_nucleation")
        d = d or (self.params["dx"],) * 3
        dt_nuc = dt_nuc if dt_nuc is not None else interval * self.params["dt"]
        check(self.L.pfa_set_nucleation_args(self.ref, interval, sigma[0], sigma[1], unit_a,
                                             d[0], d[1], d[2], dt_nuc), "pfa_set_nucleation_args")
        self.nucleation = dict(seed=int(seed), geometry=int(geometry), interval=int(interval),
                               sigma=[float(v) for v in sigma], unit_a=float(unit_a),
                               d=[float(v) for v in d], dt_nuc=float(dt_nuc))

    def checkpoint(self, path):
        """Write everything the run continues from to one .npz file: the
        fields (FP64, the reference layout, ghost ring included), the mask,
        parameters and settings, the step and nucleation-call counters and,
        for the FP32 forms, their records; Grid2D.resume(path) continues
        bit-identically."""
        import json
        steps, calls = ctypes.c_uint64(), ctypes.c_uint64()
        check(self.L.pfa_get_counters(self.ref, ctypes.byref(steps), ctypes.byref(calls)),
              "pfa_get_counters")
        fields = self.read()
        extra = {}
        nb = int(self.L.pfa_f32_state_bytes(self.ref))
        if nb:
            raw = np.empty(nb, dtype=np.uint8)
            check(self.L.pfa_read_f32_state(self.ref, raw.ctypes.data, nb), "pfa_read_f32_state")
            extra["f32_state"] = raw
        meta = dict(format=CHECKPOINT_FORMAT, dim=2, params=self.params,
                    precision=self.precision, mode=self.mode, mobility=self.mobility,
                    nucleation=self.nucleation, steps=int(steps.value),
                    nucleation_calls=int(calls.value))
        np.savez(path, cr=fields[0], nb=fields[1], pd=fields[2], pl=fields[3], mask=self.mask,
                 meta=np.array(json.dumps(meta)), **extra)

    @classmethod
    def resume(cls, path):
        """A new handle in the state a checkpoint() file holds (ValueError,
        before any device work, for a file of another format or a 3D grid)."""
        meta, fields, mask, raw = _load_checkpoint(path, dim=2)
        g = cls(fields, meta["params"], precision=meta["precision"], mode=meta["mode"],
                mask=mask, mobility=meta["mobility"])
        try:
            if meta["nucleation"]:
                g.set_nucleation(**meta["nucleation"])
            check(g.L.pfa_set_counters(g.ref, meta["steps"], meta["nucleation_calls"]),
                  "pfa_set_counters")
            if raw is not None:
                check(g.L.pfa_write_f32_state(g.ref, raw.ctypes.data, raw.size),
                      "pfa_write_f32_state")
        except BaseException:
            g.close()
            raise
        return g

    def run(self, nsteps, dt=None, alpha=None):
        dt = self.params["dt"] if dt is None else dt
        alpha = self.params["alpha"] if alpha is None else alpha
        check(self.L.pfa_run(self.ref, int(nsteps), alpha, dt), "pfa_run")

    def run_timed(self, nsteps):
        ms = ctypes.c_float()
        check(self.L.pfa_run_timed(self.ref, int(nsteps), self.params["alpha"], self.params["dt"],
                                   ctypes.byref(ms)), "pfa_run_timed")
        return ms.value

    def step_stages(self, dt=None, alpha=None):
        """One step through the reference's six stage calls + swap (src/main.cpp:289-321)."""
        dt = self.params["dt"] if dt is None else dt
        alpha = self.params["alpha"] if alpha is None else alpha
        a = (self.ref, self.nx, self.ny, 3, 13, 13)
        L = self.L
        check(L.pfa_device_boundaries(*a), "device_boundaries")
        check(L.pfa_device_fictitious(*a), "device_fictitious")
        check(L.pfa_fictitious_boundaries(*a), "fictitious_boundaries")
        check(L.pfa_device_mobilities(*a), "device_mobilities")
        check(L.pfa_mobility_boundaries(*a), "mobility_boundaries")
        check(L.pfa_device_laplacian(*a, self.params["dx"], self.params.get("dy", self.params["dx"])),
              "device_laplacian")
        check(L.pfa_device_laplacian_boundaries(*a), "device_laplacian_boundaries")
        check(L.pfa_device_evolution(*a, alpha, dt), "device_evolution")
        check(L.pfa_swap(self.ref), "swap")

    def nucleate(self, sigma=(0.13, 0.13), unit_a=0.352e-9, d=None, dt_nuc=None):
        """device_nucleation on the *_new fields (call before the swap in a manual loop)."""
        d = d or (self.params["dx"],) * 3
        check(self.L.pfa_device_nucleation(self.ref, self.nx, self.ny, 3, 13, 13, sigma[0],
                                           sigma[1], unit_a, 0.0, d[0], d[1], d[2], dt_nuc),
              "device_nucleation")

    def swap(self):
        check(self.L.pfa_swap(self.ref), "swap")

    def events(self, cap=1 << 16):
        cells = (ctypes.c_int64 * cap)()
        ph = (ctypes.c_int32 * cap)()
        n = self.L.pfa_last_nucleation_events(self.ref, cells, ph, cap)
        if n < 0:
            check(self.L.pfa_last_error(), "events")
        return [(cells[k], ph[k]) for k in range(min(n, cap))]

    def read(self, out=None, wait=True):
        """read_out_result into `out` (new arrays if None).  wait=False only
        enqueues the copies: `out` (page-locked to overlap other work) is
        filled once sync() returns."""
        out = out or [np.empty((self.ny, self.nx)) for _ in range(4)]
        fn = self.L.pfa_read_out_result if wait else self.L.pfa_read_out_result_async
        check(fn(self.ref, *[_ptr(a) for a in out], self.nx, self.ny), "read_out_result")
        return out

    def upload(self, fields, wait=True):
        """Replace the fields.  wait=False only enqueues the copies: the
        arrays must be C-contiguous float64 and stay unchanged until sync()."""
        if wait:
            f = [np.ascontiguousarray(a, dtype=np.float64) for a in fields]
            check(self.L.pfa_upload_fields(self.ref, *[_ptr(a) for a in f], self.nx, self.ny),
                  "upload_fields")
            return
        for a in fields:
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("upload(wait=False) needs C-contiguous float64 arrays")
        check(self.L.pfa_upload_fields_async(self.ref, *[_ptr(a) for a in fields], self.nx,
                                             self.ny), "upload_fields")

    def dataviz(self):
        out = [np.empty((self.ny, self.nx)) for _ in range(6)]
        check(self.L.pfa_device_dataviz(self.ref, *[_ptr(a) for a in out], self.nx, self.ny),
              "device_dataviz")
        return out

    def summarize(self):
        out = np.zeros(5)
        check(self.L.pfa_summarize(self.ref, _ptr(out)), "summarize")
        return out

    def energy(self, alpha=None, maps=False):
        """Total free energy (and the per-node chemical / gradient maps)."""
        alpha = self.params["alpha"] if alpha is None else alpha
        e = ctypes.c_double()
        chem = np.zeros((self.ny, self.nx)) if maps else None
        grad = np.zeros((self.ny, self.nx)) if maps else None
        check(self.L.pfa_summarize_energy(self.ref, self.params["dx"],
                                          self.params.get("dy", self.params["dx"]), alpha,
                                          ctypes.byref(e), _ptr(chem) if maps else None,
                                          _ptr(grad) if maps else None), "pfa_summarize_energy")
        return (e.value, chem, grad) if maps else e.value

    def sync(self):
        check(self.L.pfa_sync(self.ref), "sync")

    def close(self):
        if self._live:
            self._live = False
            check(self.L.pfa_free_cuda(self.ref), "free_cuda")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def params_vector(p):
    """The 12-double parameter block of pfa3d_create (pfa_model_params layout)."""
    return np.array(list(p["D_Cr"]) + list(p["D_Nb"]) + list(p["kappa"]) + list(p["omega"]) +
                    list(p["Lmob"]) + [p["alpha"], p["dt"]], dtype=np.float64)


class Grid3D:
    """One 3D grid (7-point Laplacian), fields (nz, ny, nx) with the ghost ring."""

    def __init__(self, fields, params, precision="fp64", recipe=None):
        """From host fields, or (fields None) built on the device from a 3D
        recipe dict (see ic_recipe)."""
        L = load()
        self.L = L
        self.params = dict(params)
        self._pv = params_vector(params)
        self._d = np.array([params["dx"], params.get("dy", params["dx"]),
                            params.get("dz", params["dx"])], dtype=np.float64)
        self.h = ctypes.c_void_p()
        if fields is None:
            self.shape = ic_shape(recipe)
            r = ic_recipe(recipe)
            check(L.pfa3d_create_ic(ctypes.byref(self.h), ctypes.byref(r), _ptr(self._pv),
                                    _ptr(self._d), PRECISIONS[precision]), "pfa3d_create_ic")
        else:
            f = [np.ascontiguousarray(a, dtype=np.float64) for a in fields]
            self.shape = f[0].shape
            nz, ny, nx = self.shape
            check(L.pfa3d_create(ctypes.byref(self.h), nx, ny, nz, _ptr(self._pv), _ptr(self._d),
                                 *[_ptr(a) for a in f], PRECISIONS[precision]), "pfa3d_create")
        self._live = True
        self.precision, self.nucleation = precision, None

    @staticmethod
    def footprint(shape, precision="fp32"):
        nz, ny, nx = shape
        return int(load().pfa3d_footprint(nx, ny, nz, PRECISIONS[precision]))

    def run(self, nsteps):
        check(self.L.pfa3d_run(self.h, int(nsteps)), "pfa3d_run")

    def run_timed(self, nsteps):
        ms = ctypes.c_float()
        check(self.L.pfa3d_run_timed(self.h, int(nsteps), ctypes.byref(ms)), "pfa3d_run_timed")
        return ms.value

    def sync(self):
        check(self.L.pfa3d_sync(self.h), "pfa3d_sync")

    def energy(self, alpha=None):
        e = ctypes.c_double()
        alpha = self.params["alpha"] if alpha is None else alpha
        check(self.L.pfa3d_summarize_energy(self.h, alpha, ctypes.byref(e)),
              "pfa3d_summarize_energy")
        return e.value

    def set_nucleation(self, seed=42, interval=0, sigma=(0.13, 0.13), unit_a=0.352e-9, d=None,
                       dt_nuc=None):
        """Nucleation after every step k with k % interval == 0 (0: off)."""
        d = d or (self.params["dx"],) * 3
        dt_nuc = dt_nuc if dt_nuc is not None else max(interval, 1) * self.params["dt"]
        check(self.L.pfa3d_set_nucleation(self.h, seed, interval, sigma[0], sigma[1], unit_a,
                                          d[0], d[1], d[2], dt_nuc), "pfa3d_set_nucleation")
        self.nucleation = dict(seed=int(seed), interval=int(interval),
                               sigma=[float(v) for v in sigma], unit_a=float(unit_a),
                               d=[float(v) for v in d], dt_nuc=float(dt_nuc))

    def checkpoint(self, path):
        """As Grid2D.checkpoint, for a 3D grid."""
        import json
        steps, calls = ctypes.c_uint64(), ctypes.c_uint64()
        check(self.L.pfa3d_get_counters(self.h, ctypes.byref(steps), ctypes.byref(calls)),
              "pfa3d_get_counters")
        fields = self.read()
        extra = {}
        nb = int(self.L.pfa3d_f32_state_bytes(self.h))
        if nb:
            raw = np.empty(nb, dtype=np.uint8)
            check(self.L.pfa3d_read_f32_state(self.h, raw.ctypes.data, nb), "pfa3d_read_f32_state")
            extra["f32_state"] = raw
        meta = dict(format=CHECKPOINT_FORMAT, dim=3, params=self.params,
                    precision=self.precision, nucleation=self.nucleation,
                    steps=int(steps.value), nucleation_calls=int(calls.value))
        np.savez(path, cr=fields[0], nb=fields[1], pd=fields[2], pl=fields[3],
                 meta=np.array(json.dumps(meta)), **extra)

    @classmethod
    def resume(cls, path):
        """A new 3D handle in the state a checkpoint() file holds (ValueError,
        before any device work, for a file of another format or a 2D grid)."""
        meta, fields, _, raw = _load_checkpoint(path, dim=3)
        g = cls(fields, meta["params"], precision=meta["precision"])
        try:
            if meta["nucleation"]:
                g.set_nucleation(**meta["nucleation"])
            check(g.L.pfa3d_set_counters(g.h, meta["steps"], meta["nucleation_calls"]),
                  "pfa3d_set_counters")
            if raw is not None:
                check(g.L.pfa3d_write_f32_state(g.h, raw.ctypes.data, raw.size),
                      "pfa3d_write_f32_state")
        except BaseException:
            g.close()
            raise
        return g

    def events(self, cap=1 << 16):
        cells = (ctypes.c_int64 * cap)()
        ph = (ctypes.c_int32 * cap)()
        n = self.L.pfa3d_last_nucleation_events(self.h, cells, ph, cap)
        if n < 0:
            check(self.L.pfa_last_error(), "events")
        return [(cells[k], ph[k]) for k in range(min(n, cap))]

    def read(self, out=None, wait=True):
        """The fields into `out` (new arrays if None); wait=False only
        enqueues the copies (`out` is filled once sync() returns)."""
        out = out or [np.empty(self.shape) for _ in range(4)]
        fn = self.L.pfa3d_read if wait else self.L.pfa3d_read_async
        check(fn(self.h, *[_ptr(a) for a in out]), "pfa3d_read")
        return out

    def upload(self, fields, wait=True):
        """Replace the fields; wait=False only enqueues the copies (C-contiguous
        float64 arrays, unchanged until sync())."""
        if wait:
            f = [np.ascontiguousarray(a, dtype=np.float64) for a in fields]
            check(self.L.pfa3d_upload(self.h, *[_ptr(a) for a in f]), "pfa3d_upload")
            return
        for a in fields:
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("upload(wait=False) needs C-contiguous float64 arrays")
        check(self.L.pfa3d_upload_async(self.h, *[_ptr(a) for a in fields]), "pfa3d_upload")

    def summarize(self):
        out = np.zeros(5)
        check(self.L.pfa3d_summarize(self.h, _ptr(out)), "pfa3d_summarize")
        return out

    def close(self):
        if self._live:
            self._live = False
            check(self.L.pfa3d_destroy(self.h), "pfa3d_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


ENOMEM = 5


class Batch:
    """Many 2D grids (FP32 form) stepped together by one launch per step.

    ``add`` returns a slot id, or None when the arena has no room for the grid
    (the admission refusal); ``remove`` frees the slot between runs."""

    def __init__(self, params, arena_bytes):
        L = load()
        self.L = L
        self.params = dict(params)
        self._pv = params_vector(params)
        self._d = np.array([params["dx"], params.get("dy", params["dx"])], dtype=np.float64)
        self.h = ctypes.c_void_p()
        check(L.pfa_batch_create(ctypes.byref(self.h), _ptr(self._pv), _ptr(self._d),
                                 int(arena_bytes)), "pfa_batch_create")
        self.shapes = {}
        self._live = True

    @staticmethod
    def footprint(shape):
        ny, nx = shape
        return int(load().pfa_batch_footprint(nx, ny))

    def add(self, fields):
        f = [np.ascontiguousarray(a, dtype=np.float64) for a in fields]
        ny, nx = f[0].shape
        slot = _i()
        rc = self.L.pfa_batch_add(self.h, nx, ny, *[_ptr(a) for a in f], ctypes.byref(slot))
        if rc == ENOMEM:
            return None
        check(rc, "pfa_batch_add")
        self.shapes[slot.value] = (ny, nx)
        return slot.value

    def add_recipe(self, rec):
        """add() with the grid built on the device from a 2D recipe dict."""
        r = ic_recipe(rec)
        slot = _i()
        rc = self.L.pfa_batch_add_ic(self.h, ctypes.byref(r), ctypes.byref(slot))
        if rc == ENOMEM:
            return None
        check(rc, "pfa_batch_add_ic")
        self.shapes[slot.value] = ic_shape(rec)
        return slot.value

    def remove(self, slot):
        check(self.L.pfa_batch_remove(self.h, slot), "pfa_batch_remove")
        self.shapes.pop(slot, None)

    def read(self, slot, out=None):
        out = out or [np.empty(self.shapes[slot]) for _ in range(4)]
        check(self.L.pfa_batch_read(self.h, slot, *[_ptr(a) for a in out]), "pfa_batch_read")
        return out

    def read_async(self, slot, out):
        """The slot's fields into `out` (four arrays, page-locked for the copy
        to be asynchronous) after the runs enqueued so far; valid after sync()."""
        check(self.L.pfa_batch_read_async(self.h, slot, *[_ptr(a) for a in out]),
              "pfa_batch_read_async")
        return out

    def run(self, nsteps):
        check(self.L.pfa_batch_run(self.h, int(nsteps)), "pfa_batch_run")

    def run_timed(self, nsteps):
        ms = ctypes.c_float()
        check(self.L.pfa_batch_run_timed(self.h, int(nsteps), ctypes.byref(ms)),
              "pfa_batch_run_timed")
        return ms.value

    def sync(self):
        check(self.L.pfa_batch_sync(self.h), "pfa_batch_sync")

    def summarize(self, slot):
        out = np.zeros(5)
        check(self.L.pfa_batch_summarize(self.h, slot, _ptr(out)), "pfa_batch_summarize")
        return out

    def tune(self, reps=10):
        ms = ctypes.c_float()
        check(self.L.pfa_batch_tune(self.h, reps, ctypes.byref(ms)), "pfa_batch_tune")
        return ms.value

    def set_launch(self, rows, persistent, ctas=0):
        check(self.L.pfa_batch_set_launch(self.h, rows, int(persistent), ctas),
              "pfa_batch_set_launch")

    def launch(self):
        v = [_i() for _ in range(4)]
        check(self.L.pfa_batch_get_launch(self.h, *[ctypes.byref(x) for x in v]),
              "pfa_batch_get_launch")
        return {"rows": v[0].value, "persistent": bool(v[1].value), "ctas": v[2].value,
                "units": v[3].value}

    def info(self):
        n, used, cap = _i(), ctypes.c_size_t(), ctypes.c_size_t()
        check(self.L.pfa_batch_info(self.h, ctypes.byref(n), ctypes.byref(used),
                                    ctypes.byref(cap)), "pfa_batch_info")
        return {"grids": n.value, "used_bytes": used.value, "arena_bytes": cap.value}

    def close(self):
        if self._live:
            self._live = False
            check(self.L.pfa_batch_destroy(self.h), "pfa_batch_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def philox_device(ctr, key):
    """Philox4x32-10 of n counters (n x 4 uint32) on the device."""
    ctr = np.ascontiguousarray(ctr, dtype=np.uint32)
    n = ctr.shape[0]
    out = np.zeros((n, 4), dtype=np.uint32)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    check(load().pfa_philox_block(ctr.ctypes.data_as(u32p), int(key), out.ctypes.data_as(u32p), n),
          "pfa_philox_block")
    return out


def split_device(v):
    """The FP32 form's split (hi, c) of an array of doubles on the device."""
    v = np.ascontiguousarray(v, dtype=np.float64).ravel()
    hi = np.zeros(v.size, dtype=np.float32)
    c = np.zeros(v.size, dtype=np.float32)
    check(load().pfa_split_block(_ptr(v), hi.ctypes.data_as(_fp), c.ctypes.data_as(_fp), v.size),
          "pfa_split_block")
    return hi, c


def fast_coef():
    out = np.zeros(44, dtype=np.float32)
    check(load().pfa_model_fast_coef(out.ctypes.data_as(_fp), 44), "pfa_model_fast_coef")
    return {"den": out[0:6], "num": out[6:30].reshape(2, 12), "dP": out[30:42].reshape(2, 6),
            "xe_gam": out[42:44]}
