"""The drop-in path the reference's driver takes, run on the GPU.

src/main.cpp:225-327 calls the library through the reference's own C++
entry points (mangled names) with a HostData of row-pointer arrays
(make_arrays, src/mesh.cpp:12-97) and swaps the CudaData's old / new device
pointers itself after every step.  Two callers replay that sequence:

* ctypes, calling the mangled symbols of libpfa_gb300.so directly with a
  HostData built here;
* tests/dropin/driver_loop.cu, the same loop in C++ compiled against
  include/pfa_reference_abi.h (its layout is checked against the reference's
  own headers in test_dropin_cpu.py).

Both are compared with the reference's own CUDA kernels run on a GB300
(tests/golden/ref_gpu_step2d.npz): FP64 within 1e-12 (per field
max|a - b| / max|b|, interior and ghost edges), the FP32 form selected with
pfa_set_precision right after init_cuda within 2e-7 absolute after 1000 steps
(the bound the form holds against FP64 there; the stated bound is 1e-5).
"""
import ctypes

import numpy as np
import pytest

from conftest import field_err, fields_of, golden, interior
from dropin import harness

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL_1000 = 2e-7

_dp = ctypes.POINTER(ctypes.c_double)
_dpp = ctypes.POINTER(_dp)
_i, _d = ctypes.c_int, ctypes.c_double

HOST_FIELDS = ("mask_lap", "conc_Ni", "phi", "chem_nrg", "grad_nrg",
               "conc_Cr_old", "conc_Cr_new", "conc_Cr_lap", "conc_Cr_gam",
               "conc_Nb_old", "conc_Nb_new", "conc_Nb_lap", "conc_Nb_gam",
               "phi_del_old", "phi_del_new", "phi_del_lap",
               "phi_lav_old", "phi_lav_new", "phi_lav_lap")


class HostData(ctypes.Structure):
    """src/type.h:28-53: row-pointer arrays over contiguous blocks."""
    _fields_ = [(n, _dpp) for n in HOST_FIELDS]


class Host:
    """A HostData with its storage: one (rows, cols) block per member and a
    row-pointer array into it, as make_arrays lays them out."""

    def __init__(self, nx, ny, nm=3):
        self.h = HostData()
        self.blocks, self._rows = {}, []
        for name in HOST_FIELDS:
            rows, cols = (nm, nm) if name == "mask_lap" else (ny, nx)
            blk = np.zeros((rows, cols))
            ptrs = (_dp * rows)(*[ctypes.cast(blk[j].ctypes.data, _dp) for j in range(rows)])
            self.blocks[name] = blk
            self._rows.append(ptrs)
            setattr(self.h, name, ctypes.cast(ptrs, _dpp))


# mangled C++ names of src/data.cuh and src/discretization.cuh (Itanium ABI)
SYMS = {
    "init_cuda": ("_Z9init_cudaP8HostDataiiiPKdS2_S2_S2_S2_P8CudaData",
                  [ctypes.c_void_p, _i, _i, _i, _dp, _dp, _dp, _dp, _dp, ctypes.c_void_p]),
    "free_cuda": ("_Z9free_cudaP8CudaData", [ctypes.c_void_p]),
    "read_out_result": ("_Z15read_out_resultP8CudaDataP8HostDataii",
                        [ctypes.c_void_p, ctypes.c_void_p, _i, _i]),
    "device_boundaries": ("_Z17device_boundariesP8CudaDataiiiii", [ctypes.c_void_p] + [_i] * 5),
    "device_fictitious": ("_Z17device_fictitiousP8CudaDataiiiii", [ctypes.c_void_p] + [_i] * 5),
    "fictitious_boundaries": ("_Z21fictitious_boundariesP8CudaDataiiiii",
                              [ctypes.c_void_p] + [_i] * 5),
    "device_laplacian": ("_Z16device_laplacianP8CudaDataiiiiidd",
                         [ctypes.c_void_p] + [_i] * 5 + [_d, _d]),
    "device_laplacian_boundaries": ("_Z27device_laplacian_boundariesP8CudaDataiiiii",
                                    [ctypes.c_void_p] + [_i] * 5),
    "device_evolution": ("_Z16device_evolutionP8CudaDataiiiiidd",
                         [ctypes.c_void_p] + [_i] * 5 + [_d, _d]),
    "device_init_prng": ("_Z16device_init_prngP8CudaDataiiiii", [ctypes.c_void_p] + [_i] * 5),
    "device_nucleation": ("_Z17device_nucleationP8CudaDataiiiiidddddddd",
                          [ctypes.c_void_p] + [_i] * 5 + [_d] * 8),
    "device_dataviz": ("_Z14device_datavizP8CudaDataP8HostDataiiiii",
                       [ctypes.c_void_p, ctypes.c_void_p] + [_i] * 5),
    "checkCuda": ("_Z9checkCuda9cudaError", [_i]),
}


def _abi(pfa):
    L = ctypes.CDLL(pfa.LIB_PATH)
    fns = {}
    for name, (sym, args) in SYMS.items():
        f = getattr(L, sym)
        f.argtypes = args
        f.restype = _i if name == "checkCuda" else None
        fns[name] = f
    return fns


def _ok(pfa, what):
    L = pfa.load()
    err = L.pfa_last_error()
    assert err == 0, f"{what}: {L.pfa_last_error_message().decode()}"


def _drive(pfa, fields, params, steps, io, precision=0, mask=None):
    """src/main.cpp's loop through the mangled entry points; returns
    {step: (dataviz arrays, read_out_result arrays)} at every output step.
    mask: the 3 x 3 Laplacian mask in host.mask_lap (default: the 5-point
    mask of src/main.cpp:237)."""
    fn = _abi(pfa)
    L = pfa.load()
    L.pfa_clear_error()
    ny, nx = fields[0].shape
    nm, bx, by = 3, 13, 13
    host = Host(nx, ny, nm)
    host.blocks["mask_lap"][:] = (pfa.five_point_mask(params["dx"], params["dx"]) if mask is None
                                  else mask)
    for name, a in zip(("conc_Cr_old", "conc_Nb_old", "phi_del_old", "phi_lav_old"), fields):
        host.blocks[name][:] = a
    consts = [np.ascontiguousarray(params[k], dtype=np.float64)
              for k in ("kappa", "omega", "Lmob", "D_Cr", "D_Nb")]
    dev = pfa.CudaData()
    hp, dp = ctypes.byref(host.h), ctypes.byref(dev)
    fn["init_cuda"](hp, nx, ny, nm, *[c.ctypes.data_as(_dp) for c in consts], dp)
    _ok(pfa, "init_cuda")
    if precision:
        pfa.check(L.pfa_set_precision(dp, precision), "pfa_set_precision")
    fn["device_init_prng"](dp, nx, ny, nm, bx, by)
    a = (dp, nx, ny, nm, bx, by)
    out = {}
    swaps = (("conc_Cr_old", "conc_Cr_new"), ("conc_Nb_old", "conc_Nb_new"),
             ("phi_del_old", "phi_del_new"), ("phi_lav_old", "phi_lav_new"))
    for k in range(steps):
        fn["device_boundaries"](*a)
        fn["device_fictitious"](*a)
        fn["fictitious_boundaries"](*a)
        fn["device_laplacian"](*a, params["dx"], params["dx"])
        fn["device_laplacian_boundaries"](*a)
        fn["device_evolution"](*a, params["alpha"], params["dt"])
        for o, n in swaps:  # the caller's swap_pointers_1D (src/main.cpp:318-321)
            # (a pointer field read from a ctypes Structure shares the
            # structure's memory: take the addresses as integers first)
            po, pn = (ctypes.cast(getattr(dev, x), ctypes.c_void_p).value for x in (o, n))
            setattr(dev, o, ctypes.cast(pn, _dp))
            setattr(dev, n, ctypes.cast(po, _dp))
        if (k + 1) % io == 0:
            fn["device_dataviz"](dp, hp, nx, ny, nm, bx, by)
            viz = [host.blocks[n].copy() for n in ("conc_Cr_new", "conc_Nb_new", "conc_Ni",
                                                   "phi_del_new", "phi_lav_new", "phi")]
            res = ("conc_Cr_new", "conc_Nb_new", "phi_del_new", "phi_lav_new")
            for n in res:
                host.blocks[n][:] = 0.0
            fn["read_out_result"](dp, hp, nx, ny)
            out[k + 1] = (viz, [host.blocks[n].copy() for n in res])
            _ok(pfa, f"output step {k + 1}")
    _ok(pfa, "step loop")
    fn["free_cuda"](dp)
    _ok(pfa, "free_cuda")
    assert not dev.conc_Cr_old and not dev.str_A, "free_cuda left pointers in CudaData"
    return out


def _check_dataviz(viz, res):
    """device_dataviz's six arrays: the fields (what read_out_result then
    copies, bit for bit), x_Ni = 1 - x_Cr - x_Nb and phi = p(phi_del) +
    p(phi_lav) (src/discretization.cu:1211-1229; phi to rounding, the device
    evaluates p with fused multiply-adds)."""
    cr, nb, ni, pd, pl, phi = viz
    for a, b in zip((cr, nb, pd, pl), res):
        assert np.array_equal(a, b)
    assert np.array_equal(ni, 1.0 - cr - nb)
    p = lambda x: x * x * x * (6.0 * x * x - 15.0 * x + 10.0)
    assert np.max(np.abs(phi - (p(pd) + p(pl)))) <= 1e-14


@pytest.mark.parametrize("caller", ["ctypes", "cxx"])
def test_fp64_driver_loop_matches_reference_kernels(pfa, tmp_path, caller):
    """The reference's own sequence of calls, FP64: the fields read back at the
    output steps equal the reference's CUDA kernels after 1, 10 and 100
    steps."""
    g = golden("step2d.npz")
    r = golden("ref_gpu_step2d.npz")
    p = pfa.model_params()
    f = fields_of(g, "ic")
    if caller == "ctypes":
        out = _drive(pfa, f, p, 10, 1)
        out.update({100: _drive(pfa, f, p, 100, 50)[100]})
    else:
        exe = harness.compile_loop(str(tmp_path))
        out = harness.run_loop(exe, str(tmp_path), f, p, 10, 1)
        out.update({100: harness.run_loop(exe, str(tmp_path), f, p, 100, 50)[100]})
    for k in (1, 10, 100):
        viz, res = out[k]
        _check_dataviz(viz, res)
        err = field_err(res, fields_of(r, f"step_s{k}"))
        assert max(err) <= FP64_TOL, (caller, k, err)


@pytest.mark.parametrize("caller", ["ctypes", "cxx"])
def test_fp32_driver_loop_matches_reference_kernels(pfa, tmp_path, caller):
    """The FP32 form behind the unchanged loop (pfa_set_precision right after
    init_cuda; the caller keeps swapping the FP64 pointers, read_out_result
    and device_dataviz export the FP32 state into whichever array is *_old):
    the 256 x 256 workload after 1000 steps, with output steps every 250
    along the way, against the reference's CUDA kernels."""
    r = golden("ref_gpu_step2d.npz")
    p = pfa.model_params()
    f = fields_of(r, "config1_ic")
    if caller == "ctypes":
        out = _drive(pfa, f, p, 1000, 250, precision=pfa.FP32)
    else:
        exe = harness.compile_loop(str(tmp_path))
        out = harness.run_loop(exe, str(tmp_path), f, p, 1000, 250, precision=pfa.FP32)
    assert sorted(out) == [250, 500, 750, 1000]
    for k in out:
        _check_dataviz(*out[k])
    err = [float(np.max(np.abs(interior(a) - interior(b))))
           for a, b in zip(out[1000][1], fields_of(r, "config1_s1000"))]
    assert max(err) <= FP32_TOL_1000, err
    # output steps do not disturb the run: the same 1000 steps without them
    g = pfa.Grid2D(f, p, precision="fp32")
    g.run(1000)
    for a, b in zip(g.read(), out[1000][1]):
        assert np.array_equal(interior(a), interior(b))
    g.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_driver_loop_with_nine_point_mask(pfa, precision):
    """The reference's loop with its 9-point mask in host.mask_lap
    (nine_point_Laplacian_stencil, src/mesh.cpp:198-213), FP64 and the FP32
    form, against the reference's CUDA kernels run with the same mask
    (tests/golden/ref_gpu_nine.npz) after 100 steps."""
    r = golden("ref_gpu_nine.npz")
    p = pfa.model_params()
    dx, dy = r["iso_dxy"]
    m9 = pfa.nine_point_mask(dx, dy)
    out = _drive(pfa, fields_of(r, "ic"), p, 100, 100,
                 precision=pfa.FP32 if precision == "fp32" else 0, mask=m9)
    _check_dataviz(*out[100])
    want = fields_of(r, "iso_s100")
    if precision == "fp64":
        assert max(field_err(out[100][1], want)) <= FP64_TOL
    else:
        err = [float(np.max(np.abs(interior(a) - interior(b)))) for a, b in zip(out[100][1], want)]
        assert max(err) <= FP32_TOL_1000, err


def test_driver_loop_with_nucleation_equals_library_loop(pfa, tmp_path):
    """device_nucleation inside the reference's loop (after device_evolution,
    before the caller's swap, every 10 steps) gives bit for bit the fields of
    the library's own multi-step loop with the same interval."""
    from golden.make_golden import NUC_A
    from pfa_gb300 import ic
    f = ic.grid2d(64, 48, seed=3, matrix=(0.2600, 0.1680), enrich=(0.2720, 0.1692),
                  stripes=[20], stripe_width=16, n_particles=1, radius=5.0)
    p = pfa.model_params()
    exe = harness.compile_loop(str(tmp_path))
    nuc = (10, NUC_A["sigma"][0], NUC_A["unit_a"], NUC_A["d"][0], NUC_A["dt"])
    out = harness.run_loop(exe, str(tmp_path), f, p, 30, 30, nuc=nuc)
    g = pfa.Grid2D(f, p)
    g.set_nucleation(seed=42, geometry=pfa.NUC_FIXED_GEOMETRY, interval=10, sigma=NUC_A["sigma"],
                     unit_a=NUC_A["unit_a"], d=NUC_A["d"], dt_nuc=NUC_A["dt"])
    g.run(30)
    want = g.read()
    g.close()
    for a, b in zip(out[30][1], want):
        assert np.array_equal(a, b, equal_nan=True)
    # nuclei were painted: the same loop without nucleation ends elsewhere
    plain = harness.run_loop(exe, str(tmp_path), f, p, 30, 30)
    assert any(not np.array_equal(a, b, equal_nan=True) for a, b in zip(out[30][1], plain[30][1]))


def test_check_cuda_reports_and_returns(pfa):
    """checkCuda (src/discretization.cu:23-30) returns its argument and
    records a failure in the error word instead of aborting."""
    fn = _abi(pfa)
    L = pfa.load()
    L.pfa_clear_error()
    assert fn["checkCuda"](0) == 0
    assert L.pfa_last_error() == 0
    assert fn["checkCuda"](2) == 2  # cudaErrorMemoryAllocation
    assert L.pfa_last_error() == 2  # PFA_ECUDA
    L.pfa_clear_error()
