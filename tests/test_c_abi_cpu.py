"""The plain-C ABI from C: a C99 program that includes only
include/pfa_gb300.h, links libpfa_gb300.so and calls the entry points that
need no GPU (model parameters, batch footprints, error strings, the refusal
of a bad argument) gets what the Python binding gets -- what a cgo or JNI
binding sees through the same header."""
import os
import subprocess

import numpy as np

from conftest import ROOT

PROGRAM = r"""
#include <stdio.h>
#include "pfa_gb300.h"

int main(void) {
  double out[13];
  int rc = pfa_model_params(5e-9, 10e-9, 0.30, 0.02, 5e-9, 2, 1, out);
  printf("rc %d\n", rc);
  for (int k = 0; k < 13; k++) printf("p%d %.17g\n", k, out[k]);
  printf("fp %zu\n", pfa_batch_footprint(130, 66));
  printf("fp0 %zu\n", pfa_batch_footprint(2, 66));
  printf("einval %s\n", pfa_error_string(PFA_EINVAL));
  /* a spacing of zero is refused on the host, with the sticky error word set */
  rc = pfa_model_params(0.0, 10e-9, 0.30, 0.02, 5e-9, 2, 1, out);
  printf("bad %d %d\n", rc, pfa_last_error());
  pfa_clear_error();
  printf("cleared %d\n", pfa_last_error());
  return 0;
}
"""


def test_c_program_links_and_matches_the_binding(pfa, tmp_path):
    src = tmp_path / "abi.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "abi"
    libdir = os.path.dirname(pfa.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-lpfa_gb300",
                    f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = dict(line.split(" ", 1) for line in out.splitlines())
    assert got["rc"] == "0"
    want = np.zeros(13)
    pfa.check(pfa.load().pfa_model_params(5e-9, 10e-9, 0.30, 0.02, 5e-9, 2, 1,
                                          pfa._ptr(want)), "pfa_model_params")
    assert [float(got[f"p{k}"]) for k in range(13)] == list(want)
    assert int(got["fp"]) == pfa.Batch.footprint((66, 130)) > 0
    assert int(got["fp0"]) == 0  # below 3 x 3 cells
    assert got["einval"] == pfa.load().pfa_error_string(1).decode()
    code, sticky = map(int, got["bad"].split())
    assert code != 0 and sticky == code
    assert got["cleared"] == "0"
