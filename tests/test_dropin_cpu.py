"""The drop-in boundary without a GPU: the reference driver's loop
(tests/dropin/driver_loop.cu) compiles and links against libpfa_gb300.so, and
the structures it sees through include/pfa_reference_abi.h have the layout
the reference's own headers give them (src/type.h:28-107).  Compiled against
the reference's src/data.cuh, src/discretization.cuh and src/type.h where the
checkout is present, so drift in a signature (a link failure) or in a
structure (a different offset) shows here."""
import pytest

from dropin import harness


def _need_nvcc():
    if not harness.nvcc():
        pytest.skip("nvcc not available")


@pytest.fixture(scope="module")
def own_loop(pfa, tmp_path_factory):
    _need_nvcc()
    return harness.compile_loop(str(tmp_path_factory.mktemp("dropin")))


def test_loop_links_against_the_library(own_loop):
    lay = harness.layout(own_loop)
    assert lay["entry_points"] == "1"
    # LP64 sizes of src/type.h's structures: 19 row-pointer members; one
    # generator pointer, 4 streams, 4 events and 16 field pointers
    assert lay["sizeof.HostData"] == str(19 * 8)
    assert lay["sizeof.CudaData"] == str(25 * 8)
    assert lay["CudaData.conc_Cr_old"] == str(11 * 8)


def test_layout_matches_the_reference_headers(own_loop, tmp_path):
    ref = harness.reference_checkout()
    if ref is None:
        pytest.skip("the reference checkout is not present")
    import os
    theirs = harness.compile_loop(str(tmp_path), ref_src=os.path.join(ref, "src"))
    assert harness.layout(theirs) == harness.layout(own_loop)
