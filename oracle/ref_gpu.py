"""The reference's own CUDA time step, launched through the CUDA driver API
(test infrastructure: the golden steps of tests/golden/make_ref_gpu_golden.py
and the reference-GPU timing leg of bench.py; the library never loads it).

oracle/Makefile's `ref-gpu` target compiles usnistgov/phasefield-precipitate-aging's
src/parabola625.cu, src/nucleation.cu and src/discretization.cu where they lie
into one sm_103a device module (oracle/_ref/ref_step.cubin; it needs the
reference checkout, so it is built in the build container and carried to the
GPU).  run_reference uploads the constants init_cuda uploads
(src/data.cu:71-80: the 5-point mask of src/mesh.cpp:187-196, D, kappa,
omega, L) and runs the reference's update loop (src/main.cpp:289-321 with
nucleation off) in its own launch order and shapes -- bx = by = 13, nm = 3
(src/main.cpp:229-231):

  device_boundaries        src/discretization.cu:396-451 (10 fields)
  device_fictitious        :128-173
  fictitious_boundaries    :453-481
  device_laplacian         :780-841 (shared tile (bx + nm) (by + nm) doubles)
  device_laplacian_boundaries :524-548
  device_evolution         :989-1020
  swap of old / new        src/main.cpp:318-321

The reference runs these on four streams ordered by events, waiting on the
host at every call; here they run in the same order on one stream without
host waits, which computes the same values (the kernels of one call touch
disjoint arrays) and is never slower.
"""
import ctypes
import os

import numpy as np

CUBIN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "ref_step.cubin")

NAMES = ("cr", "nb", "pd", "pl")
BX = BY = 13
NM = 3

# kernels of src/discretization.cu (C++ names; fp_t = double, src/type.h:23)
K_BOUNDARY = b"_Z15boundary_kernelPdiii"
K_FICT = (b"_Z21fictitious_gam_kernelPdS_S_S_S_S_iii", b"_Z21fictitious_del_kernelPdS_S_S_S_S_iii",
          b"_Z21fictitious_lav_kernelPdS_S_S_S_S_iii")
K_CONV = b"_Z18convolution_kernelPdS_iii"
K_CH = b"_Z20cahn_hilliard_kernelPdS_S_S_iiid"
K_AC = b"_Z17allen_cahn_kernelPdS_S_S_S_S_iiidd"
K_CHEM = (b"_Z30chemical_convolution_Cr_kernelPdS_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_iiidd",
          b"_Z30chemical_convolution_Nb_kernelPdS_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_iiidd")
K_INIT_PRNG = b"_Z16init_prng_kernelP17curandStateXORWOWii"
K_NUC = b"_Z17nucleation_kernelPdS_S_S_P17curandStateXORWOWiiidddddddd"
PRNG_STATE_BYTES = 64  # >= sizeof(curandStateXORWOW) (48)


class Driver:
    """The few CUDA driver calls the script needs, through ctypes."""

    def __init__(self, cubin):
        cu = ctypes.CDLL("libcuda.so.1")
        u64, sz, vp = ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p
        cu.cuModuleGetGlobal_v2.argtypes = [ctypes.POINTER(u64), ctypes.POINTER(sz), vp, ctypes.c_char_p]
        cu.cuMemAlloc_v2.argtypes = [ctypes.POINTER(u64), sz]
        cu.cuMemFree_v2.argtypes = [u64]
        cu.cuMemsetD8_v2.argtypes = [u64, ctypes.c_ubyte, sz]
        cu.cuMemcpyHtoD_v2.argtypes = [u64, vp, sz]
        cu.cuMemcpyDtoH_v2.argtypes = [vp, u64, sz]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        cu.cuLaunchKernel.argtypes = [vp] + [ctypes.c_uint] * 7 + [vp, ctypes.POINTER(vp), vp]
        self.cu = cu
        self.ck(cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self.ck(cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        self.ctx = vp()
        self.ck(cu.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self.ck(cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.mod = vp()
        self.ck(cu.cuModuleLoad(ctypes.byref(self.mod), cubin.encode()), "cuModuleLoad")
        self.fn = {}

    @staticmethod
    def ck(r, what):
        if r != 0:
            raise RuntimeError(f"{what}: CUresult {r}")

    def function(self, name):
        if name not in self.fn:
            f = ctypes.c_void_p()
            self.ck(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name), name.decode())
            self.fn[name] = f
        return self.fn[name]

    def set_constant(self, name, values):
        ptr, size = ctypes.c_uint64(), ctypes.c_size_t()
        self.ck(self.cu.cuModuleGetGlobal_v2(ctypes.byref(ptr), ctypes.byref(size), self.mod, name),
                name.decode())
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        if a.nbytes > size.value:
            raise ValueError(f"{name.decode()} holds {size.value} bytes, not {a.nbytes}")
        self.ck(self.cu.cuMemcpyHtoD_v2(ptr, a.ctypes.data, a.nbytes), "cuMemcpyHtoD")

    def alloc(self, nbytes):
        p = ctypes.c_uint64()
        self.ck(self.cu.cuMemAlloc_v2(ctypes.byref(p), nbytes), "cuMemAlloc")
        self.ck(self.cu.cuMemsetD8_v2(p, 0, nbytes), "cuMemsetD8")
        return p

    def free(self, p):
        self.ck(self.cu.cuMemFree_v2(p), "cuMemFree")

    def put(self, p, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.ck(self.cu.cuMemcpyHtoD_v2(p, a.ctypes.data, a.nbytes), "cuMemcpyHtoD")

    def get(self, p, shape):
        a = np.empty(shape, dtype=np.float64)
        self.ck(self.cu.cuMemcpyDtoH_v2(a.ctypes.data, p, a.nbytes), "cuMemcpyDtoH")
        return a

    def launch(self, name, grid, block, shmem, args):
        vals = []
        for a in args:
            if isinstance(a, ctypes.c_uint64):
                vals.append(ctypes.c_uint64(a.value))
            elif isinstance(a, int):
                vals.append(ctypes.c_int(a))
            else:
                vals.append(ctypes.c_double(a))
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p)
                                                 for v in vals])
        self.ck(self.cu.cuLaunchKernel(self.function(name), grid[0], grid[1], 1, block[0], block[1],
                                       1, shmem, None, params, None), name.decode())

    def sync(self):
        self.ck(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def close(self):
        """Unload the module and drop this object's hold on the primary context."""
        if self.mod:
            self.ck(self.cu.cuModuleUnload(self.mod), "cuModuleUnload")
            self.mod = None
            dev = ctypes.c_int()
            self.ck(self.cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
            self.ck(self.cu.cuDevicePrimaryCtxRelease(dev), "cuDevicePrimaryCtxRelease")


def n_tiles(n, tile, nm):
    """nTiles, src/discretization.cu:45-48 (float arithmetic as there)."""
    return int(np.ceil(np.float32(n) / np.float32(tile - nm + 1)))


def five_point_mask(dx, dy):
    """five_point_Laplacian_stencil, src/mesh.cpp:187-196."""
    m = np.zeros((3, 3))
    m[0][1] = 1. / (dy * dy)
    m[1][0] = 1. / (dx * dx)
    m[1][1] = -2. * (dx * dx + dy * dy) / (dx * dx * dy * dy)
    m[1][2] = 1. / (dx * dx)
    m[2][1] = 1. / (dy * dy)
    return m


def nine_point_mask(dx, dy):
    """nine_point_Laplacian_stencil, src/mesh.cpp:198-213."""
    m = np.zeros((3, 3))
    m[0][0] = 1. / (6. * dx * dy)
    m[0][1] = 4. / (6. * dy * dy)
    m[0][2] = 1. / (6. * dx * dy)
    m[1][0] = 4. / (6. * dx * dx)
    m[1][1] = -10. * (dx * dx + dy * dy) / (6. * dx * dx * dy * dy)
    m[1][2] = 4. / (6. * dx * dx)
    m[2][0] = 1. / (6. * dx * dy)
    m[2][1] = 4. / (6. * dy * dy)
    m[2][2] = 1. / (6. * dx * dy)
    return m


def _setup(drv, fields, prm, mask=None):
    """init_cuda's constant uploads and the device arrays: [old, new] fields
    and the six fictitious compositions (Cr / Nb of gamma, delta, laves).
    mask: the 3 x 3 Laplacian mask (default: the 5-point mask of prm's
    spacing, as src/main.cpp:237)."""
    ny, nx = fields[0].shape
    nb = nx * ny * 8
    drv.set_constant(b"d_mask", five_point_mask(prm.dx, prm.dy) if mask is None
                     else np.ascontiguousarray(mask, dtype=np.float64))
    for name, v in ((b"d_DCr", prm.D_Cr), (b"d_DNb", prm.D_Nb), (b"d_Kapp", prm.kappa),
                    (b"d_Omeg", prm.omega), (b"d_Lmob", prm.Lmob)):
        drv.set_constant(name, list(v))
    state = [[drv.alloc(nb) for _ in range(4)], [drv.alloc(nb) for _ in range(4)]]
    fict = [drv.alloc(nb) for _ in range(6)]
    for p, a in zip(state[0], fields):
        drv.put(p, a)
    return state, fict


def _step(drv, state, fict, nx, ny, prm):
    """One pass of src/main.cpp:289-321 (nucleation off); swaps state."""
    old, new = state
    grid = (n_tiles(nx, BX, NM), n_tiles(ny, BY, NM))
    block = (BX, BY)
    shmem = (BX + NM) * (BY + NM) * 8

    def bc(p):
        drv.launch(K_BOUNDARY, grid, block, 0, [p, nx, ny, NM])

    for p in old + fict:  # device_boundaries
        bc(p)
    for k in range(3):  # device_fictitious
        drv.launch(K_FICT[k], grid, block, 0, old + fict[2 * k:2 * k + 2] + [nx, ny, NM])
    for p in fict:  # fictitious_boundaries
        bc(p)
    for src, dst in ((old[2], new[2]), (old[3], new[3]), (fict[0], new[0]),
                     (fict[1], new[1])):  # device_laplacian
        drv.launch(K_CONV, grid, block, shmem, [src, dst, nx, ny, NM])
    for p in new:  # device_laplacian_boundaries
        bc(p)
    drv.launch(K_CH, grid, block, 0, [old[0], old[1], new[0], new[1], nx, ny, NM, prm.dt])
    drv.launch(K_AC, grid, block, 0, [old[0], old[1], old[2], old[3], new[2], new[3],
                                      nx, ny, NM, prm.alpha, prm.dt])
    state.reverse()


def run_reference(drv, fields, prm, steps, mask=None):
    """Snapshots of the reference's update loop after each count in `steps`
    (mask: the Laplacian mask, default 5-point)."""
    ny, nx = fields[0].shape
    state, fict = _setup(drv, fields, prm, mask)
    out = {}
    done = 0
    for target in steps:
        for _ in range(target - done):
            _step(drv, state, fict, nx, ny, prm)
        done = target
        drv.sync()
        out[target] = [drv.get(p, (ny, nx)) for p in state[0]]
    for p in state[0] + state[1] + fict:
        drv.free(p)
    return out


def time_reference(drv, fields, prm, steps, warmup=2):
    """Seconds per step of the reference's update loop on `fields` (warm,
    host-timed between two device synchronisations)."""
    import time
    ny, nx = fields[0].shape
    state, fict = _setup(drv, fields, prm)
    for _ in range(warmup):
        _step(drv, state, fict, nx, ny, prm)
    drv.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        _step(drv, state, fict, nx, ny, prm)
    drv.sync()
    t = (time.perf_counter() - t0) / steps
    for p in state[0] + state[1] + fict:
        drv.free(p)
    return t


def run_reference_nucleation(drv, fields, sigma, unit_a, d, dt):
    """One call of the reference's nucleation (device_init_prng, then
    nucleation_kernel on the fields, src/discretization.cu:1022-1043,1079-1177)
    with the spacing d = (dx, dy, dz) passed to the kernel as given; returns
    the fields after it.  init_prng_kernel seeds each cell's XORWOW state from
    clock(), so the draws differ from call to call: only statistics compare."""
    ny, nx = fields[0].shape
    nb = nx * ny * 8
    f = [drv.alloc(nb) for _ in range(4)]
    for p, a in zip(f, fields):
        drv.put(p, a)
    prng = drv.alloc(nx * ny * PRNG_STATE_BYTES)
    grid = (n_tiles(nx, BX, NM), n_tiles(ny, BY, NM))
    drv.launch(K_INIT_PRNG, grid, (BX, BY), 0, [prng, nx, ny])
    drv.launch(K_NUC, grid, (BX, BY), 0, f + [prng, nx, ny, NM, sigma[0], sigma[1], unit_a, 0.0,
                                              d[0], d[1], d[2], dt])
    drv.sync()
    out = [drv.get(p, (ny, nx)) for p in f]
    for p in f + [prng]:
        drv.free(p)
    return out


def run_reference_chem_div(drv, fields, fict, mob, dx, dy):
    """The reference's chemical_convolution_Cr_kernel and _Nb_kernel
    (src/discretization.cu:618-778, compiled but never launched by its loop)
    on a state: fields (x_Cr, x_Nb, phi_del, phi_lav), its six fictitious
    compositions and 16 mobility coefficients (Cr row, Nb row, in the
    kernels' argument order), in the launch shape its commented launches
    use (bx = by = 13).  Returns the two divergence arrays."""
    ny, nx = fields[0].shape
    nb = nx * ny * 8
    pf = [drv.alloc(nb) for _ in range(4)]
    pc = [drv.alloc(nb) for _ in range(6)]
    pm = [drv.alloc(nb) for _ in range(16)]
    out = [drv.alloc(nb) for _ in range(2)]
    for p, a in zip(pf + pc + pm, list(fields) + list(fict) + list(mob)):
        drv.put(p, a)
    grid = (n_tiles(nx, BX, NM), n_tiles(ny, BY, NM))
    for k in range(2):
        drv.launch(K_CHEM[k], grid, (BX, BY), 0,
                   pc + pm[8 * k:8 * k + 8] + [pf[2], pf[3], out[k], nx, ny, NM, dx, dy])
    drv.sync()
    res = [drv.get(p, (ny, nx)) for p in out]
    for p in pf + pc + pm + out:
        drv.free(p)
    return res
