// Order of the diagnostics of a geodesic (CreateDiagnosticVector, Diagnostics.cpp:14-99).
//
// The reference builds the vector in the order FourColorScreen, GeodesicPosition,
// EquatorialPasses, ClosestRadius, and appending the value diagnostic rotates the vector
// left by one. That order decides which diagnostic's value the mesh sees first
// (Geodesic.cpp:141-149), the order of the output files and of the first-line
// description (Utilities.cpp:52-84).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/foort_gpu.h"

namespace foort {

inline std::vector<uint32_t> diagnostic_order(uint32_t diag_flags, uint32_t value_diag) {
    std::vector<uint32_t> order;
    const uint32_t all[4] = {FOORT_DIAG_FOUR_COLOR_SCREEN, FOORT_DIAG_GEODESIC_POSITION, FOORT_DIAG_EQUATORIAL_PASSES,
                             FOORT_DIAG_CLOSEST_RADIUS};
    for (uint32_t f : all) {
        if (!(diag_flags & f)) continue;
        order.push_back(f);
        if (value_diag & f) std::rotate(order.begin(), order.begin() + 1, order.end());
    }
    return order;
}

}  // namespace foort
