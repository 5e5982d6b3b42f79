// Headless restatement of the reference's outer loop (src/main.cpp:538-1086)
// for the compiled reference core.  TEST INFRASTRUCTURE ONLY: it produces
// the golden record of a whole OptCuts run (dual updates, topology steps,
// fracture propagation, rollback, convergence) that the GPU outer loop is
// checked against.  The viewer and screenshot calls are dropped; the
// control flow and every numeric rule are the reference's:
//   * computeOptPicked / computeBestCand / checkCand   main.cpp:538-612
//   * updateLambda                                      main.cpp:614-618
//   * updateLambda_stationaryV (oscillation detection,
//     best-feasible record and rollback, convergence,
//     dual update, critical-lambda scheme)              main.cpp:620-884
//   * converge_preDrawFunc                              main.cpp:886-911
//   * preDrawFunc, offline, MT_OPTCUTS                  main.cpp:913-1055
#include "ref_outer.hpp"

#include "SymDirichletEnergy.hpp"
#include "TriMesh.hpp"

#include <igl/edge_lengths.h>

#include <chrono>
#include <cmath>
#include <fstream>
#include <map>
#include <vector>

extern std::vector<std::pair<double, double>> energyChanges_bSplit, energyChanges_iSplit, energyChanges_merge;
extern std::vector<std::vector<int>> paths_bSplit, paths_iSplit, paths_merge;
extern std::vector<Eigen::MatrixXd> newVertPoses_bSplit, newVertPoses_iSplit, newVertPoses_merge;
extern double filterExp_in;
extern int inSplitTotalAmt;
extern std::ofstream logFile;

namespace {

struct Outer {
    OptCuts::Optimizer* opt = nullptr;
    std::vector<double>* energyParams = nullptr;
    double upperBound = 4.1;
    const double convTol = 1.0e-3;
    bool bijective = true, rand1PInitCut = false;
    int iterNum = 0;
    int converged = 0;
    bool finished = false;
    const double fracThres = 0.0;
    const bool topoLineSearch = true;
    // critical-lambda choice handed from the dual step to the next topology step
    int opType_queried = -1;
    std::vector<int> path_queried;
    Eigen::MatrixXd newVertPos_queried;
    bool reQuery = false;
    // updateLambda_stationaryV's function-local statics
    int iterNum_bestFeasible = -1;
    OptCuts::TriMesh bestFeasible;
    double E_se_bestFeasible = __DBL_MAX__;
    int lastStationaryIterNum = 0;
    std::map<double, std::vector<std::pair<double, double>>> configs;
    // record
    std::vector<double> events;   // rows: iterNum, E_SD, E_se, lambda, nV, code

    double lam() const { return (*energyParams)[0]; }

    void record(double code)
    {
        const OptCuts::TriMesh& R = opt->getResult();
        double E_se;
        R.computeSeamSparsity(E_se);
        E_se /= R.virtualRadius;
        const double E_SD = opt->getLastEnergyVal(true) / lam();
        events.insert(events.end(), {(double)opt->getIterNum(), E_SD, E_se, 1.0 - lam(), (double)R.V_rest.rows(), code});
    }

    static int pickedSecond(const std::vector<std::pair<double, double>>& a,
                            const std::vector<std::pair<double, double>>& b, double lambda)
    {
        auto best = [lambda](const std::vector<std::pair<double, double>>& ec) {
            double m = __DBL_MAX__;
            for (const auto& e : ec) {
                if (e.first == __DBL_MAX__ || e.second == __DBL_MAX__) continue;
                m = std::min(m, e.first * (1.0 - lambda) + e.second * lambda);
            }
            return m;
        };
        return best(a) > best(b);
    }

    static int bestCand(const std::vector<std::pair<double, double>>& ec, double lambda, double& bestChange)
    {
        bestChange = __DBL_MAX__;
        int id = -1;
        for (int i = 0; i < (int)ec.size(); ++i) {
            if (ec[i].first == __DBL_MAX__ || ec[i].second == __DBL_MAX__) continue;
            const double c = ec[i].first * (1.0 - lambda) + ec[i].second * lambda;
            if (c < bestChange) {
                bestChange = c;
                id = i;
            }
        }
        return id;
    }

    static bool anyNegative(const std::vector<std::pair<double, double>>& ec)
    {
        for (const auto& e : ec)
            if (e.first < 0.0 || e.second < 0.0) return true;
        return false;
    }

    double dualUpdate(double measure) const
    {
        double l = std::max(0.0, measure - (upperBound - convTol / 2.0) + lam() / (1.0 - lam()));
        return l / (1.0 + l);
    }

    bool nearRecorded(double E_se, double lambda, double E_SD, double eps_E_se, double eps_lambda)
    {
        auto match = [&](const std::pair<const double, std::vector<std::pair<double, double>>>& row) {
            if (std::abs(row.first - E_se) >= eps_E_se) return false;
            for (const auto& l : row.second)
                if (std::abs(l.first - lambda) < eps_lambda && std::abs(l.second - E_SD) < eps_E_se) return true;
            return false;
        };
        const auto low = configs.lower_bound(E_se);
        if (low == configs.end()) return !configs.empty() && match(*configs.rbegin());
        if (low == configs.begin()) return match(*low);
        return match(*low) || match(*std::prev(low));
    }

    bool stationary(bool checkConvergence)
    {
        OptCuts::TriMesh& R = opt->getResult();
        Eigen::MatrixXd el;
        igl::edge_lengths(R.V_rest, R.F, el);
        const double eps_E_se = 1.0e-3 * el.minCoeff() / R.virtualRadius;
        const double E_SD = opt->getLastEnergyVal(true) / lam();
        double E_se;
        R.computeSeamSparsity(E_se);
        E_se /= R.virtualRadius;
        const double measure = E_SD;
        const double eps_lambda = std::min(1.0e-3, std::abs(dualUpdate(measure) - lam()));
        if (iterNum != lastStationaryIterNum) {
            const double lambda = 1.0 - lam();
            const bool osc = nearRecorded(E_se, lambda, E_SD, eps_E_se, eps_lambda);
            if (measure <= upperBound && E_se < E_se_bestFeasible) {
                iterNum_bestFeasible = iterNum;
                bestFeasible = R;
                E_se_bestFeasible = E_se;
            }
            if (osc && iterNum_bestFeasible >= 0) {
                if (iterNum_bestFeasible != iterNum) opt->setConfig(bestFeasible, iterNum, opt->getTopoIter());
                record(10);   // oscillation: converged (after a rollback)
                return false;
            }
            configs[E_se].emplace_back(lambda, E_SD);
        }
        lastStationaryIterNum = iterNum;
        if (checkConvergence && measure <= upperBound && measure >= upperBound - convTol) {
            if (iterNum_bestFeasible != iterNum) opt->setConfig(bestFeasible, iterNum, opt->getTopoIter());
            record(11);   // all converged at the bound
            return false;
        }
        (*energyParams)[0] = dualUpdate(measure);
        if (checkConvergence) {
            if (measure > upperBound) {
                if (!energyChanges_merge.empty() &&
                    pickedSecond(energyChanges_bSplit, energyChanges_merge, 1.0 - lam()) == 1)
                    do {
                        (*energyParams)[0] = dualUpdate(measure);
                    } while (pickedSecond(energyChanges_bSplit, energyChanges_merge, 1.0 - lam()) == 1);
                if (!anyNegative(energyChanges_iSplit) && !anyNegative(energyChanges_bSplit)) {
                    reQuery = true;
                }
                else {
                    double dB, dI;
                    int iB = bestCand(energyChanges_bSplit, 1.0 - lam(), dB);
                    int iI = bestCand(energyChanges_iSplit, 1.0 - lam(), dI);
                    while (dB > 0.0 && dI > 0.0) {
                        (*energyParams)[0] = dualUpdate(measure);
                        iB = bestCand(energyChanges_bSplit, 1.0 - lam(), dB);
                        iI = bestCand(energyChanges_iSplit, 1.0 - lam(), dI);
                    }
                    if (dB <= 0.0) {
                        opType_queried = 0;
                        path_queried = paths_bSplit[iB];
                        newVertPos_queried = newVertPoses_bSplit[iB];
                    }
                    else {
                        opType_queried = 1;
                        path_queried = paths_iSplit[iI];
                        newVertPos_queried = newVertPoses_iSplit[iI];
                    }
                }
            }
            else {
                bool noOp = true;
                for (const auto& e : energyChanges_merge)
                    if (e.first != __DBL_MAX__) {
                        noOp = false;
                        break;
                    }
                if (noOp) {
                    (*energyParams)[0] = 1.0 - eps_lambda;
                    opt->updateEnergyData(true, false, false);
                    if (iterNum_bestFeasible != iterNum) opt->setConfig(bestFeasible, iterNum, opt->getTopoIter());
                    record(12);   // no merge left: end
                    return false;
                }
                if (pickedSecond(energyChanges_bSplit, energyChanges_merge, 1.0 - lam()) == 0)
                    do {
                        (*energyParams)[0] = dualUpdate(measure);
                    } while (pickedSecond(energyChanges_bSplit, energyChanges_merge, 1.0 - lam()) == 0);
                double dM;
                int iM = bestCand(energyChanges_merge, 1.0 - lam(), dM);
                while (dM > 0.0) {
                    (*energyParams)[0] = dualUpdate(measure);
                    iM = bestCand(energyChanges_merge, 1.0 - lam(), dM);
                }
                opType_queried = 2;
                path_queried = paths_merge[iM];
                newVertPos_queried = newVertPoses_merge[iM];
            }
        }
        if (lam() > 1.0 - eps_lambda) (*energyParams)[0] = 1.0 - eps_lambda;
        if (lam() < eps_lambda) (*energyParams)[0] = eps_lambda;
        opt->updateEnergyData(true, false, false);
        return true;
    }

    void finish()
    {
        if (!bijective) {
            opt->setAllowEDecRelTol(false);
            converged = 0;
            opt->setPropagateFracture(false);
            while (!converged) proceed(1000);
        }
        opt->flushEnergyFileOutput();
        opt->flushGradFileOutput();
        finished = true;
    }

    void proceed(int n)
    {
        for (int i = 0; i < n && !converged; ++i) {
            converged = opt->solve(1);
            iterNum = opt->getIterNum();
        }
    }

    // one pass of preDrawFunc in offline mode
    void step()
    {
        while (!converged) proceed(1);
        const double measure = opt->getLastEnergyVal(true) / lam();
        if (converged == 2) {
            converged = 0;
            return;
        }
        if (!opt->isScaffolding() && bijective && rand1PInitCut) opt->setScaffolding(true);
        record(0);   // inner loop converged
        opt->flushEnergyFileOutput();
        opt->flushGradFileOutput();
        if (!stationary(false)) {
            finish();
            return;
        }
        if (opt->createFracture(fracThres, 0, topoLineSearch)) {
            record(1);   // boundary split or merge applied
            converged = 0;
            return;
        }
        if (measure > upperBound && opt->createFracture(fracThres, 0, topoLineSearch, true)) {
            record(2);   // interior split applied
            converged = 0;
            return;
        }
        if (!stationary(true)) {
            finish();
            return;
        }
        if (reQuery) {
            filterExp_in += std::log(2.0) / std::log(inSplitTotalAmt);
            filterExp_in = std::min(1.0, filterExp_in);
            while (!opt->createFracture(fracThres, 0, topoLineSearch, true)) {
                filterExp_in += std::log(2.0) / std::log(inSplitTotalAmt);
                filterExp_in = std::min(1.0, filterExp_in);
            }
            reQuery = false;
            record(3);   // interior split after widening the filter
        }
        else {
            opt->createFracture(opType_queried, path_queried, newVertPos_queried, topoLineSearch);
            record(4 + opType_queried);   // 4, 5, 6: critical-lambda split / interior split / merge
        }
        opType_queried = -1;
        converged = 0;
    }
};

} // namespace

RefOuterResult ref_outer_run(OptCuts::Optimizer& opt, std::vector<double>& energyParams, double upperBound,
                             bool bijective, bool rand1PInitCut, int maxSteps)
{
    Outer o;
    o.opt = &opt;
    o.energyParams = &energyParams;
    o.upperBound = upperBound;
    o.bijective = bijective;
    o.rand1PInitCut = rand1PInitCut;
    auto t0 = std::chrono::steady_clock::now();
    int steps = 0;
    while (!o.finished && steps < maxSteps) {
        o.step();
        ++steps;
    }
    RefOuterResult r;
    r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r.finished = o.finished;
    r.events = o.events;
    const OptCuts::TriMesh& R = opt.getResult();
    double E_se;
    R.computeSeamSparsity(E_se);
    r.E_se = E_se / R.virtualRadius;
    r.E_SD = opt.getLastEnergyVal(true) / energyParams[0];
    r.lambda = 1.0 - energyParams[0];
    r.iterNum = opt.getIterNum();
    r.topoIter = opt.getTopoIter();
    return r;
}
