"""Build and drive tests/dropin/driver_loop.cu, the reference driver's GPU
update loop (src/main.cpp:225-327) linked against libpfa_gb300.so through the
reference's own C++ entry points.

The reference checkout (for the variant compiled against its own headers) is
PFA_REFERENCE, else a directory named `reference` beside this repository.
"""
import os
import shutil
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(REPO, "phasefield-precipitate-aging_gb300", "pfa_gb300")
SOURCE = os.path.join(HERE, "driver_loop.cu")


def reference_checkout():
    """The reference's source tree if present (its src/type.h exists), else None."""
    ref = os.environ.get("PFA_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")
    return ref if os.path.isfile(os.path.join(ref, "src", "type.h")) else None


def nvcc():
    return shutil.which(os.environ.get("NVCC", "nvcc"))


def compile_loop(out_dir, ref_src=None):
    """Compile the harness into out_dir; against the reference's own headers
    (ref_src = its src/ directory) or include/pfa_reference_abi.h."""
    exe = os.path.join(out_dir, "driver_loop_ref" if ref_src else "driver_loop")
    cmd = [nvcc(), "-std=c++14", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", INCLUDE]
    if ref_src:
        # its discretization.cuh declares extern __constant__ symbols that this
        # whole-program build turns into local definitions (warning 20044)
        cmd += ["-DPFA_REF_HEADERS", "-I", ref_src, "-diag-suppress", "20044"]
    cmd += [SOURCE, "-o", exe, "-L", LIBDIR, "-lpfa_gb300", "-Xlinker", f"-rpath={LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return exe


def layout(exe):
    r = subprocess.run([exe, "layout"], capture_output=True, text=True, check=True)
    return dict(line.rsplit(" ", 1) for line in r.stdout.splitlines())


def write_input(path, fields, params):
    ny, nx = fields[0].shape
    with open(path, "wb") as f:
        f.write(struct.pack("<2i", nx, ny))
        for a in fields:
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
        c = ([params["dx"], params.get("dy", params["dx"])] + list(params["kappa"]) +
             list(params["omega"]) + list(params["Lmob"]) + list(params["D_Cr"]) +
             list(params["D_Nb"]) + [params["alpha"], params["dt"]])
        f.write(np.asarray(c, dtype="<f8").tobytes())


def read_output(path, nx, ny):
    """{step: (dataviz arrays x_Cr, x_Nb, x_Ni, phi_del, phi_lav, phi;
    read_out_result arrays x_Cr, x_Nb, phi_del, phi_lav)}"""
    raw = open(path, "rb").read()
    n = nx * ny * 8
    rec = 4 + 10 * n
    out = {}
    for off in range(0, len(raw), rec):
        step = struct.unpack_from("<i", raw, off)[0]
        arrs = [np.frombuffer(raw, "<f8", nx * ny, off + 4 + k * n).reshape(ny, nx)
                for k in range(10)]
        out[step] = (arrs[:6], arrs[6:])
    return out


def run_loop(exe, work, fields, params, steps, io, precision=0, nuc=None):
    """Run the loop; nuc = (interval, sigma, unit_a, dx, dt_nuc) or None."""
    ny, nx = fields[0].shape
    src, dst = os.path.join(work, "in.bin"), os.path.join(work, "out.bin")
    write_input(src, fields, params)
    cmd = [exe, "run", src, dst, str(steps), str(io), str(precision)]
    if nuc:
        cmd += [repr(float(v)) if k else str(int(v)) for k, v in enumerate(nuc)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver_loop failed ({r.returncode}):\n{r.stdout}\n{r.stderr}")
    return read_output(dst, nx, ny)
