// FOORT-side binding of the GB300 engine: one round of Main.cpp:327-414 as one engine
// call (foort_round.h).
#include "foort_round.h"

#include <string>
#include <vector>

namespace {

// The diagnostics in the order of Geodesic's diagnostic vector: CreateDiagnosticVector
// (Diagnostics.cpp:28-75) appends them in the order FourColorScreen, GeodesicPosition,
// EquatorialPasses, ClosestRadius, and appending the value diagnostic moves the vector's
// first element to its end (the value diagnostic ends up first).
std::vector<DiagBitflag> diagnostic_order(DiagBitflag all, DiagBitflag val) {
    const DiagBitflag appended[4] = {Diag_FourColorScreen, Diag_GeodesicPosition, Diag_EquatorialPasses,
                                     Diag_ClosestRadius};
    std::vector<DiagBitflag> order;
    for (DiagBitflag f : appended) {
        if (!(all & f)) continue;
        order.push_back(f);
        if (val & f) {
            order.push_back(order.front());
            order.erase(order.begin());
        }
    }
    return order;
}

}  // namespace

int IntegrateRoundOnGPU(ViewScreen* theView, GeodesicOutputHandler* out, foort_ctx* ctx, uint64_t grid,
                        DiagBitflag AllDiags, DiagBitflag ValDiag, FoortIntegrateFn integrate) {
    if (!theView || !out || !integrate || grid < 2) return FOORT_E_BADARG;
    if (AllDiags & Diag_GeodesicPosition) return FOORT_E_UNSUPPORTED;
    const largecounter n = theView->getCurNrGeodesics();
    std::vector<foort_pixel> px(n);
    std::vector<foort_result> res(n);
    for (largecounter i = 0; i < n; ++i) {
        Point pos;
        OneIndex vel;
        ScreenIndex s;
        theView->SetNewInitialConditions(i, pos, vel, s);
        px[i] = foort_pixel{0u, 0u, static_cast<uint64_t>(s[0]), static_cast<uint64_t>(s[1]), grid};
    }
    out->PrepareForOutput(n);
    const int rc = integrate(ctx, px.data(), static_cast<uint64_t>(n), res.data());
    if (rc != FOORT_OK && rc != FOORT_E_BUDGET && rc != FOORT_E_CANCELLED) return rc;
    const std::vector<DiagBitflag> order = diagnostic_order(AllDiags, ValDiag);
    for (largecounter i = 0; i < n; ++i) {
        const foort_result& r = res[i];
        std::vector<std::string> s;
        s.reserve(order.size() + 1);
        s.push_back(std::to_string(px[i].row) + " " + std::to_string(px[i].col) + " ");
        std::vector<real> values;
        for (size_t k = 0; k < order.size(); ++k) {
            real v = 0;
            if (order[k] == Diag_FourColorScreen) {
                s.push_back(std::to_string(r.quadrant));
                v = static_cast<real>(r.quadrant);
            } else if (order[k] == Diag_EquatorialPasses) {
                s.push_back(std::to_string(r.equat_passes));
                v = static_cast<real>(r.equat_passes);
            } else {
                s.push_back(std::to_string(r.closest_r));
                v = r.closest_r;
            }
            if (k == 0) values.push_back(v);  // the value diagnostic's getFinalDataVal
        }
        theView->GeodesicFinished(i, std::move(values));
        out->NewGeodesicOutput(i, std::move(s));
    }
    return rc;
}
