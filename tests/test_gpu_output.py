"""A complete FOORT run on the GPU (foort_gpu_run: engine, mesh, output files) writes
the reference's files byte for byte (-m gpu).

The two runs of the Test.cfg configuration (Johannsen, log-r, Verlet) of
tests/golden/dat: a 40^2 SimpleSquareMesh with a 1000-geodesic cache and 700 geodesics
per file, and a SquareSubdivisionMeshV2 from a 17^2 seed, whose rounds depend on the
values of the previous ones. Both kernels must reproduce every quadrant and pass count.
"""
import pytest

from foort_gb300 import abi, workloads
from test_output import RUNS, compare_dirs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("name", sorted(RUNS))
def test_run_writes_the_reference_files(engine_lib, tmp_path, name, precision):
    import foort_gb300
    foort_gb300.check_layout()
    wl = workloads.johannsen_golden(True, precision=precision)
    run = RUNS[name]
    mesh = foort_gb300.Mesh.from_spec(run["mesh"], wl.desc.diag_flags, wl.desc.value_diag)
    out = foort_gb300.Output(str(tmp_path / name), wl.desc.diag_flags, wl.desc.value_diag,
                             first_line=mesh.first_line_info(wl.desc), outputs_to_cache=run["cache"],
                             geodesics_per_file=run["per_file"])
    with foort_gb300.Engine(wl.desc) as e:
        geodesics, rounds = e.run([mesh], [out])
    out.close()
    mesh.close()
    print(f"{name}: {geodesics} geodesics in {rounds} rounds")
    compare_dirs(tmp_path, name)
