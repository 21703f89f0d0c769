"""Golden time steps from the reference's own CUDA kernels (run on a GPU).

The reference's kernels come from oracle/Makefile's `ref-gpu` target
(oracle/_ref/ref_step.cubin) and run through oracle/ref_gpu.py, which
launches them in the reference's own order and shapes (src/main.cpp:289-321,
nucleation off).  Cases, all FP64, with the inputs of tests/golden/step2d.npz
and step2d_refdt.npz and the 256 x 256 workload (ic.config1, stored with the
output: host tanh differs in the last bits between machines):

  step   : step2d.npz's grid, KKS-stable dt, snapshots after 1, 10, 100, 400 steps
  refdt  : step2d_refdt.npz's grid, the reference's own dt rule, 50 steps
  config1: 256 x 256 (one stripe, four particles), KKS-stable dt, 1000 steps

in ref_gpu_varmob.npz, the divergences of the reference's compiled (never
launched) chemical_convolution_Cr/Nb kernels on two states (step2d.npz's
grid, and the 256 x 256 workload after 1000 steps), given the fictitious
compositions and mobility coefficients of the oracle's variable-mobility
restatement (the reference's own mobility kernels are commented out);

in ref_gpu_nine.npz, the reference's step with its 9-point mask
(nine_point_Laplacian_stencil, src/mesh.cpp:198-213) on a 260 x 260 grid
with stripes and particles: snapshots after 1, 10, 100 and 500 steps at
dx = dy, and after 100 steps at dy = 1.25 dx (the nine weights then do not
sum to zero).  With that mask the Laplacian reads the ghost ring's corners,
which the reference's boundary_kernel writes from threads that race unless
each corner's writer and reader share a warp of its 13 x 13 blocks: they do
when the interior side is a multiple of 13 (260), and the script checks
that two runs agree bit for bit;

and, in ref_gpu_nucleation.npz, the event counts of the reference's own
nucleation kernel (src/discretization.cu:1079-1177, clock-seeded curand) in
four independent calls on a uniform enriched 512 x 512 grid whose nuclei
cover one cell each.

    python tests/golden/make_ref_gpu_golden.py [--cubin oracle/_ref/ref_step.cubin]
                                               [--out tests/golden/ref_gpu_step2d.npz]
                                               [--nuc-out tests/golden/ref_gpu_nucleation.npz]
                                               [--varmob-out tests/golden/ref_gpu_varmob.npz]
                                               [--nine-out tests/golden/ref_gpu_nine.npz]
                                               [--only varmob|step|nine|nucleation]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "phasefield-precipitate-aging_gb300"))

NAMES = ("cr", "nb", "pd", "pl")
# nucleation case: uniform enriched grid, P ~ 1e-3 per cell and phase
NUC_SIDE = 512
NUC_COMP = (0.2720, 0.1692)
NUC_SIGMA = (0.05, 0.06)
NUC_UNIT_A = 0.352e-9
NUC_D = (2e-9, 2e-9, 1e-3)
NUC_DT = 1e7
NUC_CALLS = 4
# 9-point case: interior side a multiple of the reference's 13-row tiles
NINE_SIDE = 260
NINE_STEPS = (1, 10, 100, 500)
NINE_ANISO_STEPS = 100


def main():
    import oracle as O
    from ref_gpu import CUBIN, Driver
    from pfa_gb300 import ic
    ap = argparse.ArgumentParser()
    ap.add_argument("--cubin", default=CUBIN)
    ap.add_argument("--out", default=os.path.join(HERE, "ref_gpu_step2d.npz"))
    ap.add_argument("--nuc-out", default=os.path.join(HERE, "ref_gpu_nucleation.npz"))
    ap.add_argument("--varmob-out", default=os.path.join(HERE, "ref_gpu_varmob.npz"))
    ap.add_argument("--nine-out", default=os.path.join(HERE, "ref_gpu_nine.npz"))
    ap.add_argument("--only", default="", choices=["", "varmob", "step", "nine", "nucleation"],
                    help="write only that set")
    args = ap.parse_args()
    drv = Driver(args.cubin)
    want = lambda k: args.only in ("", k)
    if want("varmob"):
        varmob(drv, O, args)
    if want("step"):
        steps(drv, O, ic, args)
    if want("nine"):
        nine(drv, O, ic, args)
    if want("nucleation"):
        nucleation(drv, ic, args)


def varmob(drv, O, args):
    """Divergences of the reference's chemical_convolution kernels."""
    from ref_gpu import run_reference_chem_div
    orc = O.Oracle()
    vm = {}
    states = [[np.load(os.path.join(HERE, "step2d.npz"))[f"ic_{n}"] for n in NAMES],
              [np.load(os.path.join(HERE, "ref_gpu_step2d.npz"))[f"config1_s1000_{n}"]
               for n in NAMES]]
    dxy = (5e-9, 5e-9)
    for k, st in enumerate(states):
        fict, mob = orc.mobility2d(st)
        div = run_reference_chem_div(drv, st, fict, mob, *dxy)
        for j, n in enumerate(NAMES):
            vm[f"s{k}_{n}"] = st[j]
        vm[f"s{k}_div_cr"], vm[f"s{k}_div_nb"] = div
    np.savez_compressed(args.varmob_out, dxy=np.array(dxy), **vm)
    print("reference GPU variable-mobility divergences written to", args.varmob_out)


def steps(drv, O, ic, args):
    """The reference's step with the 5-point mask."""
    from ref_gpu import run_reference
    res = {}
    g = np.load(os.path.join(HERE, "step2d.npz"))
    f = [g[f"ic_{n}"] for n in NAMES]
    for k, snap in run_reference(drv, f, O.model_params(), (1, 10, 100, 400)).items():
        for j, n in enumerate(NAMES):
            res[f"step_s{k}_{n}"] = snap[j]
    g = np.load(os.path.join(HERE, "step2d_refdt.npz"))
    f = [g[f"ic_{n}"] for n in NAMES]
    for k, snap in run_reference(drv, f, O.model_params(dt_rule=0), (50,)).items():
        for j, n in enumerate(NAMES):
            res[f"refdt_s{k}_{n}"] = snap[j]
    f = ic.config1()
    for k, snap in run_reference(drv, f, O.model_params(), (1000,)).items():
        for j, n in enumerate(NAMES):
            res[f"config1_ic_{n}"] = f[j]
            res[f"config1_s{k}_{n}"] = snap[j]
    np.savez_compressed(args.out, **res)
    print("reference GPU steps written to", args.out)


def nine(drv, O, ic, args):
    """The reference's step with its 9-point mask, two spacings."""
    from ref_gpu import nine_point_mask, run_reference
    f = ic.grid2d(NINE_SIDE, NINE_SIDE, seed=13, stripes=[60, 190], stripe_width=24,
                  n_particles=6, radius=6.0)
    res = {f"ic_{n}": f[j] for j, n in enumerate(NAMES)}
    prm = O.model_params()
    cases = (("iso", prm.dx, prm.dx, NINE_STEPS), ("aniso", prm.dx, 1.25 * prm.dx, (NINE_ANISO_STEPS,)))
    for tag, dx, dy, counts in cases:
        mask = nine_point_mask(dx, dy)
        runs = [run_reference(drv, f, prm, counts, mask=mask) for _ in range(2)]
        for k in counts:
            for j, n in enumerate(NAMES):
                a, b = runs[0][k][j], runs[1][k][j]
                if not np.array_equal(a, b):
                    raise SystemExit(f"the reference's 9-point step is not reproducible ({tag}, {k}, {n})")
                res[f"{tag}_s{k}_{n}"] = a
        res[f"{tag}_dxy"] = np.array([dx, dy])
    np.savez_compressed(args.nine_out, dt=np.array([prm.dt]), **res)
    print("reference GPU 9-point steps written to", args.nine_out)


def nucleation(drv, ic, args):
    """Event counts of the reference's nucleation kernel."""
    from ref_gpu import run_reference_nucleation
    # nucleation: event counts of the reference's own kernel on a uniform
    # enriched grid, single-cell nuclei (critical radius and scan radius
    # below one cell), independent calls
    f = ic.grid2d(NUC_SIDE, NUC_SIDE, seed=5, matrix=NUC_COMP, enrich=NUC_COMP, noise=0.0,
                  stripes=[], n_particles=0)
    counts = []
    for _ in range(NUC_CALLS):
        out = run_reference_nucleation(drv, f, NUC_SIGMA, NUC_UNIT_A, NUC_D, NUC_DT)
        counts.append([int(np.count_nonzero(out[2] == 1.0)), int(np.count_nonzero(out[3] == 1.0))])
    np.savez_compressed(args.nuc_out, counts=np.array(counts, dtype=np.int64),
                        cells=np.array([f[0].size]), comp=np.array(NUC_COMP),
                        sigma=np.array(NUC_SIGMA), unit_a=np.array([NUC_UNIT_A]),
                        d=np.array(NUC_D), dt=np.array([NUC_DT]))
    print("reference GPU nucleation counts", counts, "written to", args.nuc_out)


if __name__ == "__main__":
    main()
