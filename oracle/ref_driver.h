// ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// Interface of ref_driver.cpp for the other drivers linked with the reference's own
// translation units (shim_driver.cpp).
#pragma once

#include <cstdint>
#include <functional>

#include "Diagnostics.h"
#include "Geodesic.h"
#include "InputOutput.h"
#include "Integrators.h"
#include "Metric.h"
#include "Terminations.h"
#include "ViewScreen.h"
#include "../include/foort_gpu.h"

// Mesh description for ref_run / ref_mesh_trace / the shim test.
typedef struct ref_mesh_spec {
    int32_t kind;  // 0 SimpleSquareMesh, 1 SquareSubdivisionMeshV2
    int32_t max_subdivide;
    uint64_t total_pixels;
    uint64_t max_pixels;
    uint64_t initial_pixels;
    uint64_t iteration_pixels;
    int32_t initial_sub_to_final;
    int32_t reserved;
} ref_mesh_spec;

// The objects Main.cpp:211-235 builds, for a round body.
struct RefRunObjects {
    const Metric* metric;
    const Source* source;
    DiagBitflag diags, valdiag;
    TermBitflag terms;
    GeodesicIntegratorFunc integrator;
};

// The body of one round (Main.cpp:327-414): integrate every geodesic of the view's
// current round, report each to view->GeodesicFinished and outh->NewGeodesicOutput.
using RefRoundBody = std::function<int(ViewScreen* view, GeodesicOutputHandler* outh, const RefRunObjects& objects)>;

// A whole run of image 0 of d on mesh ms (Main.cpp:313-427) with `body` as each round's
// integration, writing the reference's output files.
int ref_run_rounds(const foort_run_desc* d, const ref_mesh_spec* ms, const char* prefix, const char* timestamp,
                   const char* ext, uint64_t to_cache, uint64_t per_file, int32_t first_line, const RefRoundBody& body,
                   uint64_t* n_geod, uint32_t* n_rounds, double* seconds);
