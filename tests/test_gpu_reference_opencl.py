"""The reference program itself on the GPU (its OpenCL host code and kernels,
built from mersenne2_gpu.cpp by oracle/build_ref.py and reaching the vendor's
OpenCL driver through oracle/ocl_min/icd_min.cpp).  Its verdicts for known
exponents show that the program timed beside this engine is the working
reference, not a broken build.  Skipped where no vendor OpenCL driver exists."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("args,verdict", [(["9941", "prp"], "2^9941 - 1 is a probable prime"),
                                          (["11213", "ll"], "2^11213 - 1 is prime"),
                                          (["9949", "prp"], "2^9949 - 1 is composite")])
def test_reference_program_on_gpu_verdicts(oracle_mod, args, verdict):
    if oracle_mod.opencl_vendor_lib() is None:
        pytest.skip("no vendor OpenCL driver on this machine")
    try:
        rc, out = oracle_mod.ref_opencl_run(args, timeout=300)
    except RuntimeError as ex:
        pytest.skip(str(ex))
    assert rc == 0, out[-2000:]
    assert "NVIDIA" in out and verdict in out, out[-2000:]
