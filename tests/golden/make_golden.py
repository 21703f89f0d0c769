"""Generate the golden vectors under tests/golden/ (run in the build container).

The vectors come from the reference's own compiled code: oracle/Makefile's
`ref` target compiles usnistgov/phasefield-precipitate-aging's
thermo/parabola625.c and thermo/nucleation.c where they lie and links them to
the oracle's step semantics (oracle/ref_shim.cpp).  The tests then pin the
oracle's restated energies and the CUDA library against these files; the
reference checkout itself is not needed to run them.

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""
import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "phasefield-precipitate-aging_gb300"))

import oracle as O  # noqa: E402
from pfa_gb300 import ic  # noqa: E402

# Nucleation parameters that give P_nuc of a few percent per cell at the
# enriched compositions (the physical ones give exactly 0): fixed geometry.
NUC_A = dict(sigma=(0.05, 0.05), unit_a=0.352e-9, d=(2e-10, 2e-10, 1.0), dt=1e6)
NUC_B = dict(sigma=(0.05, 0.05), unit_a=0.352e-9, d=(1e-10, 1e-10, 4.0), dt=1e6)


def nuc_struct(p):
    s = O.OrcNucParams()
    s.sigma[0], s.sigma[1] = p["sigma"]
    s.unit_a = p["unit_a"]
    s.dx, s.dy, s.dz = p["d"]
    s.dt = p["dt"]
    return s


def energies(ref, rng):
    n = 400
    xcr = rng.uniform(0.0, 0.6, n)
    xnb = rng.uniform(0.0, 0.3, n)
    pd = rng.uniform(0, 1, n)
    pl = rng.uniform(0, 1, n) * (1 - pd)
    pd[:25], pl[:25] = 1.0, 0.0     # pure delta
    pd[25:50], pl[25:50] = 0.0, 1.0  # pure laves
    pd[50:75], pl[50:75] = 0.0, 0.0  # pure gamma
    pg = 1 - pd - pl
    phi = rng.uniform(-0.1, 1.1, n)
    out = dict(xcr=xcr, xnb=xnb, pd=pd, pl=pl, pg=pg, phi=phi,
               p=ref.p(phi), pprime=ref.pprime(phi))
    for ph in range(3):
        for c in range(2):
            out[f"fict_{ph}_{c}"] = ref.fict(ph, c, xcr, xnb, pd, pg, pl)
        out[f"g_{ph}"] = ref.g(ph, xcr, xnb)
    mx = rng.uniform(0.05, 0.5, n)
    my = rng.uniform(0.005, 0.3, n)
    out["dx_cr"], out["dx_nb"] = mx, my
    for r in range(2):
        for c in range(2):
            out[f"D_{r}_{c}"] = ref.D(r, c, mx, my)
    # nucleation probability at enriched and matrix compositions
    nx_ = 200
    x = np.concatenate([rng.uniform(0.2473, 0.2967, nx_), rng.uniform(0.2794, 0.3288, nx_)])
    y = np.concatenate([rng.uniform(0.1659, 0.1726, nx_), rng.uniform(0.0202, 0.0269, nx_)])
    sig = np.where(np.arange(2 * nx_) % 2 == 0, 0.05, 0.13)
    dV = (2e-10) ** 2 * 1.0
    Va = 0.25 * 0.352e-9 ** 3
    R, P = [], []
    for a, b, s in zip(x, y, sig):
        dG = ref.g(0, [a], [b])[0]
        r_, p_ = ref.nucleation_probability_sphere(a, b, dG, ref.D(0, 0, [a], [b])[0],
                                                   ref.D(1, 1, [a], [b])[0], s, Va, dV / Va, dV, 1e6)
        R.append(r_)
        P.append(p_)
    out.update(nuc_x=x, nuc_y=y, nuc_sigma=sig, nuc_R=np.array(R), nuc_P=np.array(P))
    np.savez_compressed(os.path.join(HERE, "energies.npz"), **out)


def steps(ref):
    prm = O.model_params()
    f0 = ic.grid2d(30, 22, seed=11, stripe_width=10, n_particles=4, radius=4.0)
    snaps = {}
    cur = f0
    done = 0
    for k in (1, 10, 100, 400):
        cur = ref.run2d(cur, prm, k - done)
        done = k
        for j, name in enumerate(("cr", "nb", "pd", "pl")):
            snaps[f"s{k}_{name}"] = cur[j]
    np.savez_compressed(os.path.join(HERE, "step2d.npz"),
                        **{f"ic_{n}": f0[j] for j, n in enumerate(("cr", "nb", "pd", "pl"))},
                        **snaps, params=np.array([prm.dt, prm.dx]))
    # reference dt rule (stable for a particle-free grid over a short run)
    prm0 = O.model_params(dt_rule=0)
    g0 = ic.grid2d(17, 13, seed=12, stripe_width=6, n_particles=0)
    r0 = ref.run2d(g0, prm0, 50)
    np.savez_compressed(os.path.join(HERE, "step2d_refdt.npz"),
                        **{f"ic_{n}": g0[j] for j, n in enumerate(("cr", "nb", "pd", "pl"))},
                        **{f"s50_{n}": r0[j] for j, n in enumerate(("cr", "nb", "pd", "pl"))},
                        params=np.array([prm0.dt, prm0.dx]))


def nucleation(ref):
    out = {}
    for tag, p in (("a", NUC_A), ("b", NUC_B)):
        f = ic.grid2d(64, 48, seed=21, matrix=(0.2720, 0.1692), enrich=(0.2720, 0.1692),
                      stripes=[], n_particles=1, radius=5.0)
        res, events, n = ref.nucleation2d(f, nuc_struct(p), seed=42, call=0)
        for j, name in enumerate(("cr", "nb", "pd", "pl")):
            out[f"{tag}_ic_{name}"] = f[j]
            out[f"{tag}_out_{name}"] = res[j]
        out[f"{tag}_cells"] = np.array([e[0] for e in events], dtype=np.int64)
        out[f"{tag}_phases"] = np.array([e[1] for e in events], dtype=np.int32)
        out[f"{tag}_r"] = np.array([e[4] for e in events])
    np.savez_compressed(os.path.join(HERE, "nucleation.npz"), **out)


def summary(ref):
    f = ic.grid2d(40, 31, seed=31)
    np.savez_compressed(os.path.join(HERE, "summary.npz"),
                        **{f"ic_{n}": f[j] for j, n in enumerate(("cr", "nb", "pd", "pl"))},
                        summary=ref.summarize(f))


def free_energy(ref):
    """summarize_energy (src/alloy625.cpp:865-919) on a grid with particles,
    so that both the chemical and the gradient terms are exercised."""
    prm = O.model_params()
    f = ic.grid2d(40, 31, seed=32, stripe_width=10, n_particles=2, radius=4.0)
    e, chem, grad = ref.energy2d(f, prm.dx, prm.dx, list(prm.kappa), list(prm.omega), 1.07e11,
                                 maps=True)
    np.savez_compressed(os.path.join(HERE, "energy.npz"),
                        **{f"ic_{n}": f[j] for j, n in enumerate(("cr", "nb", "pd", "pl"))},
                        energy=np.array([e]), chem=chem, grad=grad,
                        params=np.array([prm.dx, prm.dx, prm.kappa[0], prm.kappa[1],
                                         prm.omega[0], prm.omega[1], 1.07e11]))


def varmob(ref):
    """The variable-mobility form with the reference's compiled energies,
    diffusivities, chemical-potential derivatives and curvatures
    (thermo/parabola625.c) through ref_shim.cpp: the derivatives at sample
    compositions, and the steps of step2d_varmob from two grids."""
    out = {}
    rng = np.random.default_rng(7)
    x = rng.uniform(0.0, 0.6, 200)
    y = rng.uniform(0.0, 0.3, 200)
    out["x"], out["y"] = x, y
    for ph in range(3):
        for c in range(2):
            out[f"dg_{ph}_{c}"] = ref.dg(ph, c, x, y)
        out[f"d2g_{ph}"] = np.array([[ref.d2g(ph, i, j) for j in range(2)] for i in range(2)])
    grids = [ic.grid2d(30, 22, seed=11, stripe_width=10, n_particles=4, radius=4.0),
             ic.grid2d(41, 37, seed=12, stripe_width=12, n_particles=2, radius=5.0)]
    p = O.model_params()
    for g, f0 in enumerate(grids):
        for j, n in enumerate(("cr", "nb", "pd", "pl")):
            out[f"g{g}_ic_{n}"] = f0[j]
        done, f = 0, f0
        for k in (1, 10, 60):
            f = ref.run2d_varmob(f, p, k - done)
            done = k
            for j, n in enumerate(("cr", "nb", "pd", "pl")):
                out[f"g{g}_s{k}_{n}"] = f[j]
        dv = ref.chem_div2d(f0, p.dx, p.dy)
        out[f"g{g}_div_cr"], out[f"g{g}_div_nb"] = dv
    out["params"] = np.array([p.dt, p.dx])
    np.savez_compressed(os.path.join(HERE, "step2d_varmob.npz"), **out)


IC_RECIPES = [
    # particles embedded with embed_OPC's box and overwrite (particle_mode 1),
    # integer centres as the reference's (MMSP grid positions), boxes inside
    # the interior; overlapping boxes test the order of embedding
    dict(nx=60, ny=44, nz=0, matrix=(0.3041, 0.0235), enrich=(0.2720, 0.1692), noise=0.002,
         seed=7, bands=[(20, 36)], dx=5e-9, width=10e-9, particle_mode=1,
         particles=[(16.0, 14.0, 0.0, 4.0, 0), (30.0, 22.0, 0.0, 5.5, 1),
                    (42.0, 28.0, 0.0, 3.0, 0)]),
    dict(nx=50, ny=50, nz=0, matrix=(0.2900, 0.0220), enrich=(0.2600, 0.1700), noise=0.0,
         seed=8, bands=[], dx=2e-9, width=10e-9, particle_mode=1,
         particles=[(25.0, 25.0, 0.0, 6.0, 1)]),
]


def initial_conditions(ref):
    """embed_OPC (src/alloy625.cpp:262-294) with the reference's compiled
    tanh_interp (thermo/nucleation.c:12-16) and p (thermo/parabola625.c),
    applied to the recipe's particle-free fields, for the recipes above; and
    tanh_interp itself on a set of distances and widths."""
    import ctypes
    out = {}
    dp = ctypes.POINTER(ctypes.c_double)
    emb = ref.lib.ref_embed_opc
    emb.restype = None
    emb.argtypes = [dp * 4] + [ctypes.c_int] * 4 + [ctypes.c_double] * 3 + [ctypes.c_int] + \
        [ctypes.c_double] * 2
    rxe = ref.lib.ref_xe  # the reference's equilibrium compositions (phase 1 delta, 2 laves)
    rxe.restype = ctypes.c_double
    rxe.argtypes = [ctypes.c_int, ctypes.c_int]
    xe = [(rxe(1, 0), rxe(1, 1)), (rxe(2, 0), rxe(2, 1))]
    for n, rec in enumerate(IC_RECIPES):
        base = dict(rec, particles=[])
        f = [np.ascontiguousarray(a) for a in O.ic_fields(base)]
        ny, nx = f[0].shape
        for (x, y, _z, R, ph) in rec["particles"]:
            emb((dp * 4)(*[a.ctypes.data_as(dp) for a in f]), nx, ny, int(x) + 1, int(y) + 1,
                xe[ph][0], xe[ph][1], R, 2 + ph, rec["dx"], rec["width"])
        for a in f:  # the recipe's ghost ring: the mirror of the interior
            ic.mirror_halo(a)
        for j, name in enumerate(("cr", "nb", "pd", "pl")):
            out[f"r{n}_{name}"] = f[j]
    ti = ref.lib.ref_tanh_interp
    ti.restype = ctypes.c_double
    ti.argtypes = [ctypes.c_double, ctypes.c_double]
    r = np.linspace(-3e-8, 3e-8, 241)
    w = np.array([2.5e-9, 5e-9, 1e-8])
    out["tanh_r"], out["tanh_w"] = r, w
    out["tanh_v"] = np.array([[ti(a, b) for a in r] for b in w])
    np.savez_compressed(os.path.join(HERE, "ic_embed.npz"), **out)


def abi_symbols(refdir):
    """Mangled names the reference's caller links against: compile a stub
    that calls every host entry point through the reference's own headers."""
    stub = os.path.join(HERE, "_abi_stub.cpp")
    with open(stub, "w") as fh:
        fh.write('#include "data.cuh"\n#include "discretization.cuh"\n'
                 "void use(HostData* h, CudaData* d, double* k) {\n"
                 "  checkCuda(cudaSuccess); init_cuda(h, 3, 3, 3, k, k, k, k, k, d);\n"
                 "  free_cuda(d); read_out_result(d, h, 3, 3); nTiles(1, 2, 3);\n"
                 "  device_fictitious(d, 1, 1, 1, 1, 1); device_boundaries(d, 1, 1, 1, 1, 1);\n"
                 "  fictitious_boundaries(d, 1, 1, 1, 1, 1);\n"
                 "  device_laplacian_boundaries(d, 1, 1, 1, 1, 1);\n"
                 "  device_laplacian(d, 1, 1, 1, 1, 1, 1.0, 1.0);\n"
                 "  device_evolution(d, 1, 1, 1, 1, 1, 1.0, 1.0);\n"
                 "  device_init_prng(d, 1, 1, 1, 1, 1);\n"
                 "  device_nucleation(d, 1, 1, 1, 1, 1, 1., 1., 1., 1., 1., 1., 1., 1.);\n"
                 "  device_dataviz(d, h, 1, 1, 1, 1, 1);\n}\n")
    obj = stub + ".o"
    subprocess.run(["nvcc", "-x", "cu", "-c", stub, "-o", obj, "-I", os.path.join(refdir, "src"),
                    "-I", os.path.join(refdir, "thermo")], check=True)
    nm = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True).stdout
    # C++ (mangled) entry points only; the CUDA runtime's own symbols have C names
    syms = sorted({ln.split()[-1] for ln in nm.splitlines() if ln.split()[-1].startswith("_Z")})
    with open(os.path.join(HERE, "reference_abi_symbols.txt"), "w") as fh:
        fh.write("\n".join(syms) + "\n")
    os.remove(stub)
    os.remove(obj)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PFA_REFERENCE") or
                    os.path.join(os.path.dirname(REPO), "reference"))
    ap.add_argument("--only", nargs="*", help="write only these sets (e.g. energy summary)")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={args.ref}"],
                   check=True)
    ref = O.load_ref()
    rng = np.random.default_rng(20261203)
    sets = {"energies": lambda: energies(ref, rng), "steps": lambda: steps(ref),
            "nucleation": lambda: nucleation(ref), "summary": lambda: summary(ref),
            "energy": lambda: free_energy(ref), "abi": lambda: abi_symbols(args.ref),
            "ic": lambda: initial_conditions(ref), "varmob": lambda: varmob(ref)}
    for name, fn in sets.items():
        if not args.only or name in args.only:
            fn()
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
