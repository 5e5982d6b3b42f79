// Headless restatement of the reference's outer loop (src/main.cpp:538-1086);
// test infrastructure only (see ref_outer.cpp).
#pragma once

#include "Optimizer.hpp"

#include <vector>

struct RefOuterResult {
    bool finished = false;
    double E_SD = 0.0, E_se = 0.0, lambda = 0.0, seconds = 0.0;
    int iterNum = 0, topoIter = 0;
    // one row per outer event: Newton iteration count, E_SD, E_se, lambda,
    // vertex count, event code (0 inner loop converged, 1 boundary split or
    // merge, 2 interior split, 3 interior split after widening the filter,
    // 4/5/6 critical-lambda boundary split / interior split / merge,
    // 10 oscillation, 11 converged at the bound, 12 no merge left)
    std::vector<double> events;
};

// Runs preDrawFunc's offline loop (MT_OPTCUTS) until converge_preDrawFunc
// or maxSteps passes.
RefOuterResult ref_outer_run(OptCuts::Optimizer& opt, std::vector<double>& energyParams, double upperBound,
                             bool bijective, bool rand1PInitCut, int maxSteps);
