"""FOORT .cfg files read as the reference reads them (Config.cpp:94-1155).

The strongest pin: the reference's own Test.cfg gives the first line of the reference's
shipped output files (FOORT/Output/Test_*.dat). The other tests cover libconfig's syntax,
its typed lookups without automatic conversion, and every default and fallback of the
reference's settings code, on configurations written here.
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from foort_gb300 import abi

import oracle  # noqa: E402  (only for the location of the reference's sources)

REF_CFG = oracle.REF_SRC


def load(text):
    import foort_gb300
    return foort_gb300.load_config(text=text)


@pytest.mark.skipif(not os.path.isdir(REF_CFG), reason="the reference's configuration files are not here")
def test_shipped_test_cfg_gives_the_shipped_first_line(engine_lib):
    import foort_gb300
    cfg, notes = foort_gb300.load_config(os.path.join(REF_CFG, "Test.cfg"))
    assert notes == []
    mesh = foort_gb300.config_mesh(cfg)
    header = str(np.load(os.path.join(GOLDEN, "johannsen_test.npz"))["passes_header"])
    assert mesh.first_line_info(cfg.run) == header
    assert cfg.file_prefix == b"Output/Test" and cfg.file_extension == b"dat" and cfg.timestamp == 0
    assert cfg.outputs_to_cache == 2000000 and cfg.geodesics_per_file == 2000000 and cfg.first_line_info == 1
    mesh.close()


@pytest.mark.skipif(not os.path.isdir(REF_CFG), reason="the reference's configuration files are not here")
def test_shipped_test2_cfg(engine_lib):
    import foort_gb300
    cfg, notes = foort_gb300.load_config(os.path.join(REF_CFG, "Test2.cfg"))
    d = cfg.run
    assert d.metric_id == abi.METRIC_KERR and cfg.image.metric_params[0] == 0.99 and d.rlog == 0
    assert d.diag_flags == abi.DIAG_GEODESIC_POSITION and d.value_diag == abi.DIAG_GEODESIC_POSITION
    assert d.geopos_output_steps == 5000
    # SphereRadius = 1000 is an integer: the double lookup fails, the default (1000) stays
    assert d.boundary_radius == 1000.0 and d.timeout_max_steps == 1000000
    assert cfg.mesh_kind == abi.CONFIG_MESH_INPUT_PIXELS and cfg.total_pixels == 14745600
    with pytest.raises(foort_gb300.FoortError):
        foort_gb300.config_mesh(cfg)  # pixels typed on the console: not in the engine


def test_empty_file_gives_every_default(engine_lib):
    cfg, notes = load("")
    d, im = cfg.run, cfg.image
    assert d.metric_id == abi.METRIC_KERR and im.metric_params[0] == 0.5 and d.rlog == 0
    assert d.diag_flags == d.value_diag == abi.DIAG_FOUR_COLOR_SCREEN
    assert d.term_flags == abi.TERM_BOUNDARY_SPHERE | abi.TERM_TIMEOUT
    assert d.boundary_radius == 1000.0 and d.timeout_max_steps == 10000
    assert list(im.cam_pos) == [0.0, 1000.0, 3.1415926535 / 2.0, 0.0] and list(im.cam_dir) == [0.0, -1.0, 0.0, 0.0]
    assert list(im.screen_size) == [10.0, 10.0] and list(im.screen_center) == [0.0, 0.0]
    assert cfg.mesh_kind == abi.CONFIG_MESH_SIMPLE and cfg.total_pixels == 10000
    assert d.integrator_id == abi.INTEGRATOR_RK4 and d.epsilon == 0.03 and d.smallest_step == 1e-12
    assert d.derivative_h == 1e-7 and d.verlet_tol == 0.001
    assert cfg.file_prefix == b""  # console output
    assert len(notes) >= 5


def test_typed_lookups_without_conversion(engine_lib):
    cfg, notes = load("""
        Metric = { Name = "KERR"; a = 1; RLogScale = 1; };   // integer a, integer RLogScale
        Diagnostics = { ClosestRadius = { On = true; UseForMesh = true; } };
        Terminations = { TimeOut = { On = true; MaxSteps = 5000000000; UpdateFrequency = -3; };
                         BoundarySphere = { On = true; SphereRadius = 500.; } };
        Integrator = { Type = "verlet"; StepSize = 1e-2; VerletVelocityTolerance = 0; };
    """)
    d = cfg.run
    assert d.metric_id == abi.METRIC_KERR and cfg.image.metric_params[0] == 0.5  # a = 1 is not a double
    assert d.rlog == 0  # RLogScale = 1 is not a boolean
    assert any("a" in n for n in notes)
    assert d.timeout_max_steps == 5000000000  # beyond 32 bits: a 64-bit integer
    assert d.timeout_every == 0  # negative int read as unsigned: 0
    assert d.boundary_radius == 500.0
    assert d.integrator_id == abi.INTEGRATOR_VERLET and d.epsilon == 0.01
    assert d.verlet_tol == 0.001  # 0 is an integer: the default stays
    assert d.diag_flags == d.value_diag == abi.DIAG_CLOSEST_RADIUS


def test_syntax(engine_lib):
    cfg, notes = load("""
        # comments of all three kinds /* and : assignment
        Metric : { Name = "Johann" "sen"; a = 0.5; alpha13 = -1.5e0; RLogScale = TRUE; }
        /* a block
           comment */
        ViewScreen = { Position = { r = 50.0, theta = 1.2; }; Mesh = { Type = "SimpleSquareMesh"; TotalPixels = 0x40L; } };
        Terminations = { Horizon = { On = true; }, TimeOut = { On = true; MaxSteps = 20; } };
        Diagnostics = { EquatorialPasses = { On = true; UseForMesh = true; Threshold = 0.02;
                                             UpdateFrequency = 0; UpdateStart = false; } ;
                        FourColorScreen = { On = true; UseForMesh = true; } };
        Lists = ( 1, "two", [3.0, 4.0], { x = 1; } );
    """)
    d, im = cfg.run, cfg.image
    assert d.metric_id == abi.METRIC_JOHANNSEN and d.rlog == 1
    assert list(im.metric_params[:5]) == [0.5, -1.5, 0.0, 0.0, 0.0]
    assert im.cam_pos[1] == 50.0 and im.cam_pos[2] == 1.2 and im.cam_pos[0] == 0.0
    assert cfg.total_pixels == 64
    assert d.term_flags == abi.TERM_HORIZON | abi.TERM_TIMEOUT and d.horizon_eps == 0.01 and d.timeout_max_steps == 20
    # UseForMesh is taken in the order FourColorScreen, GeodesicPosition, EquatorialPasses
    assert d.value_diag == abi.DIAG_FOUR_COLOR_SCREEN
    assert d.equat_threshold == 0.02
    assert (d.equat_freq.every_n, d.equat_freq.at_start, d.equat_freq.at_finish) == (0, 0, 1)


def test_fallbacks(engine_lib):
    # flat space has no horizon: the Horizon termination is dropped (Config.cpp:649-657)
    cfg, notes = load('Metric = { Name = "FlatSpace"; }; Terminations = { Horizon = { On = true; } };')
    assert cfg.run.metric_id == abi.METRIC_FLAT
    assert cfg.run.term_flags == abi.TERM_BOUNDARY_SPHERE | abi.TERM_TIMEOUT  # then none: the defaults
    # diagnostics on but none for the mesh and no FourColorScreen: the default diagnostic
    cfg, _ = load("Diagnostics = { ClosestRadius = { On = true; } };")
    assert cfg.run.diag_flags == cfg.run.value_diag == abi.DIAG_FOUR_COLOR_SCREEN
    # V2 mesh: MaxPixels below InitialPixels is raised to it; MaxSubdivide < 1 becomes 1
    cfg, notes = load('ViewScreen = { Mesh = { Type = "SquareSubdivisionMeshV2"; InitialPixels = 400; '
                      'MaxPixels = 0; IterationPixels = 50; MaxSubdivide = 0; InitialSubdivisionToFinal = true; } };')
    assert cfg.mesh_kind == abi.CONFIG_MESH_SUBDIVISION_V2
    assert (cfg.initial_pixels, cfg.max_pixels, cfg.iteration_pixels, cfg.max_subdivide) == (400, 400, 50, 1)
    assert cfg.initial_sub_to_final == 1
    # an unknown integrator keeps the step sizes read before the type
    cfg, _ = load('Integrator = { Type = "Euler"; StepSize = 0.1; SmallestPossibleStepsize = 1e-9; };')
    assert cfg.run.integrator_id == abi.INTEGRATOR_RK4 and cfg.run.epsilon == 0.1 and cfg.run.smallest_step == 1e-9
    # output: per-file 0 means unlimited, timestamp on by default
    cfg, _ = load('Output = { FilePrefix = "out/run"; GeodesicsPerFile = 0; GeodesicsToCache = 0; };')
    assert cfg.file_prefix == b"out/run" and cfg.timestamp == 1 and cfg.first_line_info == 1
    assert cfg.geodesics_per_file == 2 ** 64 - 1 and cfg.outputs_to_cache == 0
    # unknown metric name: default Kerr
    cfg, notes = load('Metric = { Name = "Schwarzschild"; };')
    assert cfg.run.metric_id == abi.METRIC_KERR and cfg.image.metric_params[0] == 0.5 and notes


def test_parse_errors(engine_lib):
    import foort_gb300
    for bad in ("Metric = { a = 0.5; a = 0.6; };", "Metric = { a = ; };", 'Metric = { Name = "Kerr ; };',
                "Metric = { a = 0.5;", "@include \"x.cfg\"", "x = 1.2.3;"):
        with pytest.raises(foort_gb300.FoortError):
            load(bad)
    with pytest.raises(foort_gb300.FoortError) as e:
        foort_gb300.load_config("/nonexistent/config.cfg")
    assert e.value.code == abi.FOORT_E_IO


def test_timestamp_format(engine_lib):
    import ctypes as C
    import foort_gb300
    buf = C.create_string_buffer(32)
    assert foort_gb300.load().foort_timestamp_string(buf, len(buf)) == 0
    s = buf.value.decode()
    assert len(s) == 13 and s[6] == "-" and (s[:6] + s[7:]).isdigit()


def test_default_theta_is_the_reference_pi(engine_lib):
    cfg, _ = load("")
    assert cfg.image.cam_pos[2] != math.pi / 2 and cfg.image.cam_pos[2] == 3.1415926535 / 2
