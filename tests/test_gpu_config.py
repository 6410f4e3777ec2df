"""A FOORT run from a .cfg file on the GPU writes the reference's files (-m gpu).

The configuration below is the Test.cfg configuration (Johannsen a = 0.7, alpha13 = 2,
log-r, Verlet without velocity iterations, all four terminations) on a 40^2
SimpleSquareMesh, caching 1000 geodesics and writing 700 per file: the run of
tests/golden/dat/simple40_*. Config -> engine -> files must give those files byte for byte.
"""
import pytest

from foort_gb300 import abi
from test_output import compare_dirs

pytestmark = pytest.mark.gpu

CFG = """
Metric = { Name = "Johannsen"; a = 0.7; alpha13 = 2.0; alpha22 = 0.0; alpha52 = 0.; epsilon3 = 0.; RLogScale = true; };
Diagnostics = {
    FourColorScreen = { On = true; UseForMesh = false; };
    EquatorialPasses = { On = true; UseForMesh = true; };
};
Terminations = {
    Horizon = { On = true; Epsilon_Horizon = 0.3; };
    BoundarySphere = { On = true; SphereRadius = 1000.0; };
    TimeOut = { On = true; MaxSteps = 10000; };
    ThetaSingularity = { On = true; Epsilon = 1e-5; };
};
ViewScreen = {
    Position = { t = 0.0; r = 1000.0; theta = 0.087266462599716478846; phi = 0.0; }
    Direction = { t = 0.0; r = -1.0; theta = 0.0; phi = 0.0; }
    ScreenSize = { x = 15.0; y = 15.0; }
    ScreenCenter = { x = 0.0; y = 0.0; }
    Mesh = { Type = "SimpleSquareMesh"; TotalPixels = 1600; }
};
Source = { Name = "NoSource"; };
Integrator = { Type = "Verlet"; VerletVelocityTolerance = -1.0; StepSize = 0.03; SmallestPossibleStepsize = 1e-7; };
Output = { FilePrefix = "%s"; FileExtension = "dat"; TimeStamp = false; GeodesicsToCache = 1000;
           GeodesicsPerFile = 700; FirstLineInfo = true; };
"""


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_config_run_writes_the_reference_files(engine_lib, tmp_path, precision):
    import foort_gb300
    path = tmp_path / "run.cfg"
    path.write_text(CFG % str(tmp_path / "simple40"))
    geodesics, rounds, notes = foort_gb300.run_config(str(path), precision=precision)
    assert (geodesics, rounds) == (1600, 1) and notes == []
    compare_dirs(tmp_path, "simple40")
