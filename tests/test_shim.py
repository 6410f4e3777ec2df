"""The engine's FOORT-side binding (foort_gb300/shim/foort_round.cpp) inside the
reference's own program.

oracle/Makefile builds the binding against the reference's headers and links it with the
reference's ViewScreen, Mesh and GeodesicOutputHandler objects (compiled from its
sources) and with libfoort_gpu.so, as a FOORT program would be built. The reference's
round loop (Main.cpp:313-427) then runs FOORT/Test.cfg with IntegrateRoundOnGPU as each
round's body, and the files its GeodesicOutputHandler writes must be the shipped
FOORT/Output/Test_*.dat, byte for byte. Without a GPU the binding's engine call is the
oracle (foort_gpu_integrate's contract on the CPU); the GPU's own results through the same
C ABI are compared with the reference's files in test_gpu_output.py and
test_gpu_config.py. Only where the reference's sources exist.
"""
import ctypes as C
import os

import pytest

import oracle
from foort_gb300 import abi, workloads


@pytest.fixture(scope="module")
def shim_lib(engine_lib):
    if not os.path.isdir(oracle.REF_SRC):
        pytest.skip("the reference's sources are not on this machine")
    oracle.build(with_ref=True)
    lib = C.CDLL(os.path.join(oracle.HERE, "_ref", "libfoort_shim.so"))
    lib.shim_run.argtypes = [C.POINTER(abi.RunDesc), C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint64,
                             C.c_uint64, C.c_int32, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
    return lib


def test_binding_in_the_reference_program_writes_the_shipped_files(shim_lib, tmp_path):
    wl = workloads.johannsen_golden(True)
    spec = oracle.RefMeshSpec(0, 1, 250 * 250, 0, 0, 0, 0, 0)
    prefix = os.path.join(str(tmp_path), "Test")
    n, r = C.c_uint64(), C.c_uint32()
    rc = shim_lib.shim_run(C.byref(wl.desc), C.byref(spec), prefix.encode(), b"", b"dat", 1 << 40, 1 << 40, 1,
                           os.cpu_count() or 1, C.byref(n), C.byref(r))
    assert rc == 0 and n.value == 62500 and r.value == 1
    for diag in ("EquatPasses", "FourColorScreen"):
        got = (tmp_path / f"Test_{diag}.dat").read_bytes()
        with open(os.path.join(oracle.REF_SRC, "Output", f"Test_{diag}.dat"), "rb") as f:
            want = f.read()
        assert got == want, diag


def test_binding_runs_an_adaptive_mesh_like_the_reference(shim_lib, tmp_path):
    """A V2 mesh (5 rounds on a 17^2 seed): the binding's values drive the reference's
    own mesh, so its rounds and files equal those of the reference's loop."""
    wl = workloads.johannsen_golden(False)
    wl.desc.timeout_max_steps = 20000
    spec = oracle.RefMeshSpec(1, 3, 0, 0, 17 * 17, 150, 0, 0)
    a, b = os.path.join(str(tmp_path), "shim"), os.path.join(str(tmp_path), "ref")
    n1, r1, n2, r2 = C.c_uint64(), C.c_uint32(), C.c_uint64(), C.c_uint32()
    assert shim_lib.shim_run(C.byref(wl.desc), C.byref(spec), a.encode(), b"", b"dat", 1 << 40, 1 << 40, 1,
                             os.cpu_count() or 1, C.byref(n1), C.byref(r1)) == 0
    secs = C.c_double()
    assert oracle.ref_lib().ref_run(C.byref(wl.desc), C.byref(spec), b.encode(), b"", b"dat", 1 << 40, 1 << 40, 1,
                                    os.cpu_count() or 1, C.byref(n2), C.byref(r2), C.byref(secs)) == 0
    assert (n1.value, r1.value) == (n2.value, r2.value) and r1.value > 1
    for diag in ("EquatPasses", "FourColorScreen"):
        assert (tmp_path / f"shim_{diag}.dat").read_bytes() == (tmp_path / f"ref_{diag}.dat").read_bytes(), diag
