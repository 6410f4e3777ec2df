// FOORT-side binding of the GB300 engine (include/foort_gpu.h).
//
// This file and foort_round.cpp are compiled INTO a FOORT program: they include FOORT's
// own headers (ViewScreen.h, InputOutput.h, Diagnostics.h) and replace the body of its
// round loop, the OpenMP loop of Main.cpp:327-414 that integrates every geodesic of the
// current round, with one call to the engine. FOORT's ViewScreen, Mesh and
// GeodesicOutputHandler stay as they are. Link with -lfoort_gpu -lcudart.
//
// Main.cpp's loop then reads
//     while (!theView->IsFinished()) {
//         IntegrateRoundOnGPU(theView.get(), &theOutputHandler, ctx, grid, AllDiags, ValDiag);
//         theView->EndCurrentLoop();
//     }
#pragma once

#include <cstdint>

#include "Diagnostics.h"
#include "InputOutput.h"
#include "ViewScreen.h"
#include "foort_gpu.h"

// The engine call that integrates a round's pixels: foort_gpu_integrate, or any function
// of its signature and contract.
typedef int (*FoortIntegrateFn)(foort_ctx* ctx, const foort_pixel* px, uint64_t n, foort_result* out);

// One round of a FOORT run on the engine:
//   - the round's pixels: theView->SetNewInitialConditions(i, ...) for every index (only
//     the screen index is kept; the engine forms the initial conditions itself), with
//     `grid` the mesh's R, so that the unit screen point is (row, col) / (R - 1);
//   - out->PrepareForOutput(n), then one call integrate(ctx, px, n, results);
//   - for every geodesic, theView->GeodesicFinished(i, values) and
//     out->NewGeodesicOutput(i, strings), as Main.cpp:399-400 do: values is what
//     Geodesic::getDiagnosticFinalValue gives (Geodesic.cpp:141-149), strings what
//     Geodesic::getAllOutputStr gives (Geodesic.cpp:111-139): "row col " and then every
//     diagnostic's getFullDataStr (Diagnostics.cpp:202-206, 383-387, 448-452) in the order
//     of the diagnostic vector (CreateDiagnosticVector, Diagnostics.cpp:28-75).
// Returns FOORT_OK, the engine's error code (FOORT_E_BUDGET and FOORT_E_CANCELLED still
// deliver the round, with the stopped geodesics' partial records), or
// FOORT_E_UNSUPPORTED when GeodesicPosition is among the diagnostics: its positions come
// from a second engine pass (foort_gpu_positions), which foort_gpu_run makes itself.
int IntegrateRoundOnGPU(ViewScreen* theView, GeodesicOutputHandler* out, foort_ctx* ctx, uint64_t grid,
                        DiagBitflag AllDiags, DiagBitflag ValDiag, FoortIntegrateFn integrate = foort_gpu_integrate);
