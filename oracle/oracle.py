"""ctypes front-end of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It loads ``oracle/liboracle.so`` (built by
``oracle/Makefile``) and, when present, ``oracle/_ref/libpfa_ref.so`` (the
reference's own energy functions linked to the same step semantics).

Fields are numpy float64 arrays shaped (ny, nx) or (nz, ny, nx) in the
reference's halo layout (one ghost cell on every side).  Field order:
x_Cr, x_Nb, phi_delta, phi_laves.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_dbl_p = ctypes.POINTER(ctypes.c_double)


class OrcParams(ctypes.Structure):
    _fields_ = [("D_Cr", ctypes.c_double * 2), ("D_Nb", ctypes.c_double * 2),
                ("kappa", ctypes.c_double * 2), ("omega", ctypes.c_double * 2),
                ("Lmob", ctypes.c_double * 2), ("alpha", ctypes.c_double),
                ("dt", ctypes.c_double), ("dx", ctypes.c_double),
                ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("mask3", ctypes.c_int), ("mask9", ctypes.c_double * 9)]

    def as_dict(self):
        return {"D_Cr": list(self.D_Cr), "D_Nb": list(self.D_Nb),
                "kappa": list(self.kappa), "omega": list(self.omega),
                "Lmob": list(self.Lmob), "alpha": self.alpha, "dt": self.dt,
                "dx": self.dx, "dy": self.dy, "dz": self.dz}

    def with_mask(self, mask):
        """A copy whose 2D step convolves the 3 x 3 `mask` as given (the
        reference's convolution_kernel) instead of the 5-point mask."""
        p = OrcParams.from_buffer_copy(self)
        p.mask3 = 1
        for k, w in enumerate(np.asarray(mask, dtype=np.float64).ravel()):
            p.mask9[k] = w
        return p

    @classmethod
    def from_dict(cls, d):
        p = cls()
        for k in ("D_Cr", "D_Nb", "kappa", "omega", "Lmob"):
            getattr(p, k)[0] = d[k][0]
            getattr(p, k)[1] = d[k][1]
        for k in ("alpha", "dt", "dx", "dy", "dz"):
            setattr(p, k, d[k])
        return p


class OrcNucParams(ctypes.Structure):
    _fields_ = [("sigma", ctypes.c_double * 2), ("unit_a", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("dz", ctypes.c_double), ("dt", ctypes.c_double)]


class OrcNucEvent(ctypes.Structure):
    _fields_ = [("cell", ctypes.c_int64), ("phase", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("xcr", ctypes.c_double),
                ("xnb", ctypes.c_double), ("r_precip", ctypes.c_double)]


def build(fast=True, ref=False):
    """Compile the oracle with make (cheap no-op when up to date)."""
    targets = ["liboracle.so"] + (["liboracle_fast.so"] if fast else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _ptr(a):
    return a.ctypes.data_as(_dbl_p)


class Oracle:
    """One loaded oracle library; prefix 'orc_' (restated) or 'ref_' (reference energies)."""

    def __init__(self, path=None, prefix="orc_"):
        if path is None:
            path = os.path.join(HERE, "liboracle.so")
            if not os.path.exists(path):
                build(fast=False)
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        L, P = self.lib, prefix
        d, i = ctypes.c_double, ctypes.c_int
        self._p = getattr(L, P + "p")
        self._p.restype, self._p.argtypes = d, [d]
        self._pp = getattr(L, P + "pprime")
        self._pp.restype, self._pp.argtypes = d, [d]
        self._fict = getattr(L, P + "fict")
        self._fict.restype, self._fict.argtypes = d, [i, i, d, d, d, d, d]
        self._g = getattr(L, P + "g")
        self._g.restype, self._g.argtypes = d, [i, d, d]
        self._D = getattr(L, P + "D")
        self._D.restype, self._D.argtypes = d, [i, i, d, d]
        self._nuc = getattr(L, P + "nucleation_probability_sphere")
        self._nuc.restype = None
        self._nuc.argtypes = [d] * 10 + [_dbl_p, _dbl_p]
        self._step2d = getattr(L, P + "step2d")
        self._step2d.restype = None
        self._step2d.argtypes = [ctypes.POINTER(_dbl_p), ctypes.POINTER(_dbl_p), i, i,
                                 ctypes.POINTER(OrcParams), _dbl_p]
        self._run2d = getattr(L, P + "run2d")
        self._run2d.restype = None
        self._run2d.argtypes = [ctypes.POINTER(_dbl_p), ctypes.POINTER(_dbl_p), i, i,
                                ctypes.POINTER(OrcParams), _dbl_p, i]
        self._run2d_vm = getattr(L, P + "run2d_varmob")
        self._run2d_vm.restype = None
        self._run2d_vm.argtypes = [ctypes.POINTER(_dbl_p), ctypes.POINTER(_dbl_p), i, i,
                                   ctypes.POINTER(OrcParams), _dbl_p, i]
        self._mob2d = getattr(L, P + "mobility2d")
        self._mob2d.restype = None
        self._mob2d.argtypes = [ctypes.POINTER(_dbl_p), i, i, ctypes.POINTER(_dbl_p),
                                ctypes.POINTER(_dbl_p)]
        self._cdiv = getattr(L, P + "chem_div2d")
        self._cdiv.restype = None
        self._cdiv.argtypes = [ctypes.POINTER(_dbl_p), i, i, d, d, ctypes.POINTER(_dbl_p)]
        self._dg = getattr(L, P + ("dg" if P == "orc_" else "dg_phase"))
        self._dg.restype, self._dg.argtypes = d, [i, i, d, d]
        self._d2g = getattr(L, P + ("d2g" if P == "orc_" else "d2g_phase"))
        self._d2g.restype, self._d2g.argtypes = d, [i, i, i]
        self._step3d = getattr(L, P + "step3d")
        self._step3d.restype = None
        self._step3d.argtypes = [ctypes.POINTER(_dbl_p), ctypes.POINTER(_dbl_p), i, i, i,
                                 ctypes.POINTER(OrcParams), _dbl_p]
        self._nuc2d = getattr(L, P + "nucleation2d")
        self._nuc2d.restype = i
        self._nuc2d.argtypes = [ctypes.POINTER(_dbl_p), i, i, ctypes.POINTER(OrcNucParams),
                                ctypes.c_uint64, ctypes.c_uint64,
                                ctypes.POINTER(OrcNucEvent), i]
        self._sum2d = getattr(L, P + "summarize2d")
        self._sum2d.restype = None
        self._sum2d.argtypes = [ctypes.POINTER(_dbl_p), i, i, _dbl_p]
        self._sum3d = getattr(L, P + "summarize3d")
        self._sum3d.restype = None
        self._sum3d.argtypes = [ctypes.POINTER(_dbl_p), i, i, i, _dbl_p]
        self._energy2d = getattr(L, P + "energy2d")
        self._energy2d.restype = ctypes.c_double
        self._energy2d.argtypes = [ctypes.POINTER(_dbl_p), i, i, ctypes.c_double, ctypes.c_double,
                                   _dbl_p, _dbl_p, ctypes.c_double, _dbl_p, _dbl_p]

    # ---- pointwise (vectorised by np.frompyfunc-free loops: small inputs only) ----
    def p(self, x):
        return np.array([self._p(float(v)) for v in np.ravel(x)])

    def pprime(self, x):
        return np.array([self._pp(float(v)) for v in np.ravel(x)])

    def fict(self, phase, comp, xcr, xnb, pd, pg, pl):
        return np.array([self._fict(phase, comp, *map(float, t))
                         for t in zip(xcr, xnb, pd, pg, pl)])

    def g(self, phase, xcr, xnb):
        return np.array([self._g(phase, float(a), float(b)) for a, b in zip(xcr, xnb)])

    def D(self, row, col, xcr, xnb):
        return np.array([self._D(row, col, float(a), float(b)) for a, b in zip(xcr, xnb)])

    def nucleation_probability_sphere(self, xcr, xnb, dG, dcc, dnn, sigma, vatom, n_gam, dV, dt):
        R, P = ctypes.c_double(), ctypes.c_double()
        self._nuc(xcr, xnb, dG, dcc, dnn, sigma, vatom, n_gam, dV, dt,
                  ctypes.byref(R), ctypes.byref(P))
        return R.value, P.value

    # ---- whole-grid operations ----
    @staticmethod
    def _arr4(fields):
        arrs = [np.ascontiguousarray(f, dtype=np.float64) for f in fields]
        return arrs, (_dbl_p * 4)(*[_ptr(a) for a in arrs])

    def run2d(self, fields, params, nsteps, threads=None):
        """nsteps steps from `fields` (list of 4 (ny, nx) arrays, copied); returns new list."""
        a = [np.array(f, dtype=np.float64, copy=True) for f in fields]
        b = [np.empty_like(x) for x in a]
        ny, nx = a[0].shape
        work = np.empty(2 * nx * ny, dtype=np.float64)
        pa = (_dbl_p * 4)(*[_ptr(x) for x in a])
        pb = (_dbl_p * 4)(*[_ptr(x) for x in b])
        prm = params if isinstance(params, OrcParams) else OrcParams.from_dict(params)
        self._run2d(pa, pb, nx, ny, ctypes.byref(prm), _ptr(work), int(nsteps))
        by_addr = {x.ctypes.data: x for x in a + b}
        return [by_addr[ctypes.cast(pa[k], ctypes.c_void_p).value] for k in range(4)]

    def run2d_varmob(self, fields, params, nsteps):
        """run2d with the variable-mobility Cahn-Hilliard (step2d_varmob)."""
        a = [np.array(f, dtype=np.float64, copy=True) for f in fields]
        b = [np.empty_like(x) for x in a]
        ny, nx = a[0].shape
        work = np.empty(22 * nx * ny, dtype=np.float64)
        pa = (_dbl_p * 4)(*[_ptr(x) for x in a])
        pb = (_dbl_p * 4)(*[_ptr(x) for x in b])
        prm = params if isinstance(params, OrcParams) else OrcParams.from_dict(params)
        self._run2d_vm(pa, pb, nx, ny, ctypes.byref(prm), _ptr(work), int(nsteps))
        by_addr = {x.ctypes.data: x for x in a + b}
        return [by_addr[ctypes.cast(pa[k], ctypes.c_void_p).value] for k in range(4)]

    def mobility2d(self, fields):
        """(fict[6], mob[16]) of a state: x_gam, x_del, x_lav (Cr, Nb) and the
        Cr and Nb rows of the mobility coefficients, ghost ring mirrored."""
        f = [np.ascontiguousarray(x, dtype=np.float64) for x in fields]
        ny, nx = f[0].shape
        fict = [np.zeros((ny, nx)) for _ in range(6)]
        mob = [np.zeros((ny, nx)) for _ in range(16)]
        self._mob2d((_dbl_p * 4)(*[_ptr(x) for x in f]), nx, ny,
                    (_dbl_p * 6)(*[_ptr(x) for x in fict]), (_dbl_p * 16)(*[_ptr(x) for x in mob]))
        return fict, mob

    def chem_div2d(self, fields, dx, dy):
        """The variable-mobility divergences (Cr, Nb) at the interior cells."""
        f = [np.ascontiguousarray(x, dtype=np.float64) for x in fields]
        ny, nx = f[0].shape
        out = [np.zeros((ny, nx)) for _ in range(2)]
        self._cdiv((_dbl_p * 4)(*[_ptr(x) for x in f]), nx, ny, dx, dy,
                   (_dbl_p * 2)(*[_ptr(x) for x in out]))
        return out

    def dg(self, phase, comp, x, y):
        return np.array([self._dg(phase, comp, float(a), float(b))
                         for a, b in zip(np.ravel(x), np.ravel(y))])

    def d2g(self, phase, i, j):
        return self._d2g(phase, i, j)

    def run3d(self, fields, params, nsteps):
        a = [np.array(f, dtype=np.float64, copy=True) for f in fields]
        b = [np.empty_like(x) for x in a]
        nz, ny, nx = a[0].shape
        work = np.empty(2 * nx * ny * nz, dtype=np.float64)
        prm = params if isinstance(params, OrcParams) else OrcParams.from_dict(params)
        for _ in range(int(nsteps)):
            pa = (_dbl_p * 4)(*[_ptr(x) for x in a])
            pb = (_dbl_p * 4)(*[_ptr(x) for x in b])
            self._step3d(pa, pb, nx, ny, nz, ctypes.byref(prm), _ptr(work))
            a, b = b, a
        return a

    def nucleation2d(self, fields, nuc, seed, call, max_events=1 << 16):
        """Applies nucleation in place on a copy; returns (fields, events list)."""
        a = [np.array(f, dtype=np.float64, copy=True) for f in fields]
        ny, nx = a[0].shape
        pa = (_dbl_p * 4)(*[_ptr(x) for x in a])
        ev = (OrcNucEvent * max_events)()
        n = self._nuc2d(pa, nx, ny, ctypes.byref(nuc), seed, call, ev, max_events)
        events = [(ev[k].cell, ev[k].phase, ev[k].xcr, ev[k].xnb, ev[k].r_precip)
                  for k in range(min(n, max_events))]
        return a, events, n

    def nucleation3d(self, fields, nuc, seed, call, max_events=1 << 16):
        """3D form of nucleation2d (spheres)."""
        a = [np.array(f, dtype=np.float64, copy=True) for f in fields]
        nz, ny, nx = a[0].shape
        pa = (_dbl_p * 4)(*[_ptr(x) for x in a])
        ev = (OrcNucEvent * max_events)()
        fn = getattr(self.lib, self.prefix + "nucleation3d")
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.POINTER(_dbl_p), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                       ctypes.POINTER(OrcNucParams), ctypes.c_uint64, ctypes.c_uint64,
                       ctypes.POINTER(OrcNucEvent), ctypes.c_int]
        n = fn(pa, nx, ny, nz, ctypes.byref(nuc), seed, call, ev, max_events)
        events = [(ev[k].cell, ev[k].phase, ev[k].xcr, ev[k].xnb, ev[k].r_precip)
                  for k in range(min(n, max_events))]
        return a, events, n

    def energy2d(self, fields, dx, dy, kappa, omega, Omega, maps=False):
        """Total free energy (and the per-node chemical / gradient maps),
        src/alloy625.cpp:752-807,865-919."""
        arrs, pa = self._arr4(fields)
        ny, nx = arrs[0].shape
        k = np.ascontiguousarray(kappa, dtype=np.float64)
        w = np.ascontiguousarray(omega, dtype=np.float64)
        chem = np.zeros((ny, nx)) if maps else None
        grad = np.zeros((ny, nx)) if maps else None
        e = self._energy2d(pa, nx, ny, dx, dy, _ptr(k), _ptr(w), Omega,
                           _ptr(chem) if maps else None, _ptr(grad) if maps else None)
        return (e, chem, grad) if maps else e

    def summarize(self, fields):
        arrs, pa = self._arr4(fields)
        out = np.zeros(5)
        if arrs[0].ndim == 2:
            ny, nx = arrs[0].shape
            self._sum2d(pa, nx, ny, _ptr(out))
        else:
            nz, ny, nx = arrs[0].shape
            self._sum3d(pa, nx, ny, nz, _ptr(out))
        return out


def model_params(dx=5e-9, ifce_width=10e-9, xcr0=0.30, xnb0=0.02, meshres=None,
                 dim=2, dt_rule=1, lib=None):
    """Model parameters of src/main.cpp:252-268 (meshres defaults to dx).

    dt_rule 1 (default): half the KKS-aware explicit stability limit;
    dt_rule 0: the reference's own dt formula."""
    if lib is None:
        lib = Oracle()
    f = lib.lib.orc_model_params_rule
    f.restype = None
    f.argtypes = [ctypes.c_double] * 5 + [ctypes.c_int, ctypes.c_int, ctypes.POINTER(OrcParams)]
    p = OrcParams()
    f(dx, ifce_width, xcr0, xnb0, dx if meshres is None else meshres, dim, dt_rule,
      ctypes.byref(p))
    return p


class OrcIcRecipe(ctypes.Structure):
    """orc_ic_recipe (pfa_oracle.h)."""
    _d, _i = ctypes.c_double, ctypes.c_int
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i),
                ("matrix", _d * 2), ("enrich", _d * 2), ("noise", _d), ("seed", ctypes.c_uint64),
                ("n_bands", _i), ("band", (_i * 2) * 16),
                ("n_particles", _i), ("centre", (_d * 3) * 64),
                ("radius", _d * 64), ("phase", _i * 64),
                ("dx", _d), ("width", _d), ("profile", _i), ("bell_sigma", _d * 2),
                ("bell_range", _d * 2), ("bell_x0", _d), ("particle_mode", _i)]


def ic_fields(rec, lib=None):
    """The four fields of a recipe dict (nx, ny, nz, matrix, enrich, noise,
    seed, bands [(lo, hi)], particles [(x, y, z, radius, phase)], dx, width),
    with the ghost ring."""
    if lib is None:
        lib = Oracle()
    r = OrcIcRecipe()
    r.nx, r.ny, r.nz = int(rec["nx"]), int(rec["ny"]), int(rec.get("nz", 0))
    r.matrix[:] = rec["matrix"]
    r.enrich[:] = rec["enrich"]
    r.noise, r.seed = rec["noise"], int(rec["seed"])
    bands, parts = rec.get("bands", []), rec.get("particles", [])
    r.n_bands, r.n_particles = len(bands), len(parts)
    for k, (lo, hi) in enumerate(bands):
        r.band[k][0], r.band[k][1] = int(lo), int(hi)
    for k, (x, y, z, rad, ph) in enumerate(parts):
        r.centre[k][0], r.centre[k][1], r.centre[k][2] = x, y, z
        r.radius[k], r.phase[k] = rad, int(ph)
    r.dx, r.width = rec["dx"], rec["width"]
    r.profile = int(rec.get("profile", 0))
    r.bell_sigma[:] = rec.get("bell_sigma", (0.0, 0.0))
    r.bell_range[:] = rec.get("bell_range", (0.0, 0.0))
    r.bell_x0 = rec.get("bell_x0", 0.0)
    r.particle_mode = int(rec.get("particle_mode", 0))
    shape = ((r.nz + 2, r.ny + 2, r.nx + 2) if r.nz > 1 else (r.ny + 2, r.nx + 2))
    out = [np.zeros(shape) for _ in range(4)]
    f = lib.lib.orc_ic_fields
    f.restype = None
    f.argtypes = [ctypes.POINTER(OrcIcRecipe), ctypes.POINTER(_dbl_p)]
    f(ctypes.byref(r), (_dbl_p * 4)(*[_ptr(a) for a in out]))
    return out


def philox(ctr, key, lib=None):
    if lib is None:
        lib = Oracle()
    f = lib.lib.orc_philox4x32_10
    f.restype = None
    u32 = ctypes.c_uint32
    f.argtypes = [ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u32)]
    c = (u32 * 4)(*ctr)
    k = (u32 * 2)(*key)
    o = (u32 * 4)()
    f(c, k, o)
    return list(o)


def load_ref():
    """The reference-energy variant (build container only)."""
    path = os.path.join(HERE, "_ref", "libpfa_ref.so")
    if not os.path.exists(path):
        return None
    return Oracle(path, prefix="ref_")
