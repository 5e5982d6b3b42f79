// The OptCuts outer loop on top of the library's own entry points: the
// inner Newton loop with fracture propagation, the dual (lambda) update
// with oscillation detection, best-feasible rollback and the convergence
// test, and the topology steps between inner loops.
//
// Reference: src/main.cpp:538-1086 (computeOptPicked, computeBestCand,
// checkCand, updateLambda, updateLambda_stationaryV, converge_preDrawFunc,
// preDrawFunc for the offline MT_OPTCUTS method), src/Optimizer.cpp:203-261
// (solve: propagation after each Newton iteration), :373-503
// (createFracture, both forms), src/TriMesh.cpp:760-1052 (splitEdge,
// mergeEdge, splitOrMerge).
//
// Every query runs batched on the device (oc_topology_queries /
// oc_topology_query_tail); every Newton iteration is oc_optimizer_solve.
// The host keeps only the control state the reference keeps in main.cpp's
// globals and function-local statics, and the candidate lists of the last
// queries (energyChanges_*, paths_*, newVertPoses_*) that the critical-lambda
// scheme re-ranks.
#include "optcuts_gpu.h"

#include <algorithm>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <map>
#include <new>
#include <string>
#include <vector>

namespace {

enum { kBSplit = 0, kISplit = 1, kMerge = 2 };

struct Cand {
    double ec0 = 0.0, ec1 = 0.0;
    std::vector<int> path;
    std::vector<double> pos;
};

// a recorded result mesh (the reference copies its TriMesh)
struct Snapshot {
    int nV = 0, nF = 0, nCohE = 0;
    std::vector<double> Vrest, UV;
    std::vector<int> F, cohE;
    int tails[3] = {-1, -1, -1};
};

double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

} // namespace

struct oc_optcuts {
    oc_optimizer* opt = nullptr;
    oc_mesh* mesh = nullptr;
    oc_optcuts_config cfg;
    double upperBound = 4.1;
    const double convTol = 1.0e-3;   // convTol_upperBound (main.cpp:61)
    int iterNum = 0, converged = 0, topoIter = 0;
    bool finished = false;
    int propagate = 0;               // Optimizer::propagateFracture
    bool lastPropagate = false;      // Optimizer::solve's static
    double filterExp = 0.6;          // filterExp_in
    int inSplitTotalAmt = 0;
    double virtualRadius = 1.0;
    std::vector<Cand> lists[3];      // energyChanges / paths / newVertPoses of the last queries
    int opType_queried = -1;
    Cand queried;
    bool reQuery = false;
    // updateLambda_stationaryV's statics
    int iterNum_bestFeasible = -1;
    Snapshot bestFeasible;
    double E_se_bestFeasible = DBL_MAX;
    int lastStationaryIterNum = 0;
    std::map<double, std::vector<std::pair<double, double>>> configs;
    // record
    std::vector<double> events;   // rows: Newton iterations, E_SD, E_se, lambda, vertices, event code
    std::vector<double> trace;    // rows: Newton iterations, E_w, E_SD, E_se, lambda, vertices, ||g||^2
    double ms[4] = {0, 0, 0, 0};  // Newton, queries, operations, total
    int rc = OC_OK;               // first error met
    std::vector<int> initSeams;   // TriMesh::initSeams: the cohesive edges of the initial cut
    std::vector<float> featX, featT;   // recorded (features, target) pairs

    // ---- state access -------------------------------------------------
    double lam()
    {
        double p = 0.0;
        oc_optimizer_get_energy_param(opt, &p);
        return p;
    }
    void setLam(double p) { keep(oc_optimizer_set_energy_param(opt, p)); }
    bool keep(int r)
    {
        if (r != OC_OK && rc == OC_OK) rc = r;
        return r == OC_OK;
    }
    double energySD()   // getLastEnergyVal(true) / energyParams[0]
    {
        double e = 0.0, es = 0.0;
        keep(oc_optimizer_get_last_energy(opt, &e));
        keep(oc_optimizer_get_last_energy_scaffold(opt, &es));
        return (e - es) / lam();
    }
    double seam()   // computeSeamSparsity / virtualRadius
    {
        double s = 0.0;
        keep(oc_mesh_seam_length(mesh, &s));
        return s / virtualRadius;
    }
    int nVerts()
    {
        int n = 0;
        keep(oc_mesh_get_topology(mesh, &n, nullptr, nullptr, nullptr, nullptr, nullptr));
        return n;
    }
    void record(double code)
    {
        events.insert(events.end(), {(double)iterNum, energySD(), seam(), 1.0 - lam(), (double)nVerts(), code});
    }
    void traceRow()
    {
        const double sd = energySD(), se = seam(), l = lam();
        double gsq = 0.0;
        keep(oc_optimizer_last_step(opt, nullptr, nullptr, nullptr, nullptr, &gsq));
        trace.insert(trace.end(),
                     {(double)iterNum, l * sd + (1.0 - l) * se, sd, se, 1.0 - l, (double)nVerts(), gsq});
    }
    Snapshot snapshot()
    {
        Snapshot s;
        keep(oc_mesh_get_topology(mesh, &s.nV, &s.nF, &s.nCohE, nullptr, nullptr, nullptr));
        s.Vrest.resize(3 * (size_t)s.nV);
        s.UV.resize(2 * (size_t)s.nV);
        s.F.resize(3 * (size_t)s.nF);
        s.cohE.resize(4 * (size_t)s.nCohE);
        keep(oc_mesh_get_topology(mesh, nullptr, nullptr, nullptr, s.F.data(), s.Vrest.data(), s.cohE.data()));
        keep(oc_mesh_get_uv(mesh, s.UV.data()));
        keep(oc_mesh_fracture_tails(mesh, s.tails));
        return s;
    }
    void setConfig(const Snapshot& s)   // Optimizer::setConfig(config, iterNum, topoIter)
    {
        keep(oc_optimizer_set_state(opt, s.nV, s.Vrest.data(), s.UV.data(), s.nF, s.F.data(), s.nCohE,
                                    s.cohE.data(), s.tails, iterNum));
    }
    double minEdgeLen()   // igl::edge_lengths(V_rest, F).minCoeff()
    {
        int nV = 0, nF = 0;
        keep(oc_mesh_get_topology(mesh, &nV, &nF, nullptr, nullptr, nullptr, nullptr));
        std::vector<double> Vr(3 * (size_t)nV);
        std::vector<int> F(3 * (size_t)nF);
        keep(oc_mesh_get_topology(mesh, nullptr, nullptr, nullptr, F.data(), Vr.data(), nullptr));
        double m = DBL_MAX;
        for (int t = 0; t < nF; ++t)
            for (int k = 0; k < 3; ++k) {
                const double* a = &Vr[3 * (size_t)F[3 * t + (k + 1) % 3]];
                const double* b = &Vr[3 * (size_t)F[3 * t + (k + 2) % 3]];
                m = std::min(m, std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                                          (a[2] - b[2]) * (a[2] - b[2])));
            }
        return m;
    }

    // ---- queries and operations --------------------------------------
    static void readList(const oc_topo_result* r, std::vector<Cand>& out)
    {
        int n = 0;
        oc_topo_result_info(r, &n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
        out.assign(n, Cand());
        for (int c = 0; c < n; ++c) {
            int pl = 0, pr = 0;
            double ec[2];
            oc_topo_result_candidate(r, c, nullptr, ec, nullptr, &pl, nullptr, &pr);
            out[c].ec0 = ec[0];
            out[c].ec1 = ec[1];
            out[c].path.resize(pl);
            out[c].pos.resize(2 * (size_t)pr);
            oc_topo_result_candidate(r, c, nullptr, nullptr, out[c].path.data(), nullptr, out[c].pos.data(), nullptr);
        }
    }
    // EwDec_max of a query and its best candidate (querySplit returns 0 when
    // no vertex passes its filter, TriMesh.cpp:601-604, 618-621)
    // the Optimizer's scaffolding is on (Optimizer::isScaffolding); the
    // reference's TriMesh then has a scaffold and its queries are bijective
    bool scafOn() const { return oc_optimizer_get_scaffold(opt, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr) == OC_OK; }
    int queryOptions() const
    {
        return cfg.topoOptions | (cfg.recordFeatures && !cfg.mlp ? OC_TOPO_RECORD_FEATURES : 0) |
               (cfg.bijective && scafOn() ? OC_TOPO_BIJECTIVE : 0);
    }
    // `scaffold = Scaffold(result, ...)` after a step (Optimizer.cpp:241-257)
    void rebuildScaffold()
    {
        if (!scafOn()) return;
        const auto t0 = std::chrono::steady_clock::now();
        keep(oc_optimizer_rebuild_scaffold(opt));
        ms[0] += ms_since(t0);
    }
    void keepFeatures(const oc_topo_result* r)
    {
        if (!cfg.recordFeatures || cfg.mlp) return;
        int n = 0;
        if (oc_topo_result_features(r, &n, nullptr, nullptr, nullptr) || n <= 0) return;
        const size_t x0 = featX.size(), t0 = featT.size();
        featX.resize(x0 + 32 * (size_t)n);
        featT.resize(t0 + n);
        keep(oc_topo_result_features(r, &n, featX.data() + x0, featT.data() + t0, nullptr));
    }
    static double bestOf(const oc_topo_result* r, bool split, Cand* best)
    {
        int n = 0, b = -1, pool = 0;
        oc_topo_result_info(r, &n, &b, &pool, nullptr, nullptr, nullptr, nullptr);
        if (split && pool == 0) return 0.0;
        if (b < 0) return -DBL_MAX;
        double ew = -DBL_MAX;
        int pl = 0, pr = 0;
        oc_topo_result_candidate(r, b, &ew, nullptr, nullptr, &pl, nullptr, &pr);
        if (best) {
            best->path.resize(pl);
            best->pos.resize(2 * (size_t)pr);
            oc_topo_result_candidate(r, b, nullptr, nullptr, best->path.data(), nullptr, best->pos.data(), nullptr);
        }
        return ew;
    }
    bool apply(int op, const Cand& c)
    {
        const auto t0 = std::chrono::steady_clock::now();
        const bool ok = keep(oc_optimizer_create_fracture(opt, op, c.path.data(), (int)c.path.size(), c.pos.data(),
                                                          (int)(c.pos.size() / 2)));
        ms[2] += ms_since(t0);
        return ok;
    }

    // Optimizer::createFracture(stressThres, propType, allowPropagate,
    // allowInSplit) (Optimizer.cpp:440-503)
    bool createFracture(double thres, int propType, bool allowPropagate, bool allowInSplit = false)
    {
        if (propType == 0) ++topoIter;
        const double lt = 1.0 - lam();
        const auto t0 = std::chrono::steady_clock::now();
        bool changed = false, isMerge = false;
        Cand pick;
        int pickOp = -1;
        double best = -DBL_MAX;
        if (propType == 0) {
            // TriMesh::splitOrMerge (TriMesh.cpp:978-1052)
            if (allowInSplit) {
                const int op = kISplit;
                oc_topo_result* r = nullptr;
                if (!keep(oc_topology_queries(mesh, &op, 1, lt, filterExp, queryOptions(), cfg.mlp, cfg.topFrac, &r)))
                    return false;
                keepFeatures(r);
                readList(r, lists[kISplit]);
                oc_topo_result_info(r, nullptr, nullptr, &inSplitTotalAmt, nullptr, nullptr, nullptr, nullptr);
                best = bestOf(r, true, &pick);
                pickOp = kISplit;
                oc_topo_result_destroy(r);
            }
            else {
                const int ops[2] = {kBSplit, kMerge};
                oc_topo_result* r[2] = {};
                if (!keep(oc_topology_queries(mesh, ops, 2, lt, filterExp, queryOptions(), cfg.mlp, cfg.topFrac, r)))
                    return false;
                keepFeatures(r[0]);
                keepFeatures(r[1]);
                readList(r[0], lists[kBSplit]);
                readList(r[1], lists[kMerge]);
                Cand cs, cm;
                const double es = bestOf(r[0], true, &cs), em = bestOf(r[1], false, &cm);
                if (em > es) {   // the larger decrease, split on ties (TriMesh.cpp:1002-1013)
                    isMerge = true;
                    best = em;
                    pick = cm;
                    pickOp = kMerge;
                }
                else {
                    best = es;
                    pick = cs;
                    pickOp = kBSplit;
                }
                oc_topo_result_destroy(r[0]);
                oc_topo_result_destroy(r[1]);
            }
        }
        else {
            // propagation at the fracture tail: TriMesh::splitEdge /
            // mergeEdge with propagate = true (TriMesh.cpp:760-799, 951-976)
            const int op = propType == 1 ? kBSplit : kMerge;
            isMerge = propType == 2;
            oc_topo_result* r = nullptr;
            if (!keep(oc_topology_query_tail(mesh, op, lt,
                                             cfg.topoOptions | (cfg.bijective && scafOn() ? OC_TOPO_BIJECTIVE : 0),
                                             &r)))
                return false;
            best = bestOf(r, false, &pick);
            pickOp = op;
            oc_topo_result_destroy(r);
        }
        ms[1] += ms_since(t0);
        if (best > thres && !pick.path.empty()) changed = apply(pickOp, pick);
        if (changed && allowPropagate && propType == 0) propagate = 1 + (isMerge ? 1 : 0);
        return changed;
    }

    // Optimizer::createFracture(opType, path, newVertPos, allowPropagate)
    // (Optimizer.cpp:373-438)
    bool createFracture(int opType, const Cand& c, bool allowPropagate)
    {
        ++topoIter;
        const bool ok = apply(opType, c);
        if (ok && allowPropagate) propagate = 1 + (opType == kMerge ? 1 : 0);
        return ok;
    }

    // Optimizer::solve(1) (Optimizer.cpp:203-261): 1 converged or stopped,
    // 2 a propagation run ended, 0 otherwise
    int solve1()
    {
        const auto t0 = std::chrono::steady_clock::now();
        int res = 0;
        const int r = oc_optimizer_solve(opt, 1, &res);
        ms[0] += ms_since(t0);
        if (r != OC_OK && r != OC_ERR_NOT_CONVERGED) {
            keep(r);
            return 1;
        }
        keep(oc_optimizer_get_iter_num(opt, &iterNum));
        traceRow();
        if (res == 1) return 1;
        if (propagate > 0) {
            double eDec = 0.0;
            keep(oc_optimizer_last_edec(opt, &eDec));
            if (!createFracture(eDec, propagate, true)) {
                rebuildScaffold();   // (an applied operation rebuilt it already)
                if (lastPropagate) {
                    lastPropagate = false;
                    return 2;
                }
            }
            else {
                lastPropagate = true;
            }
        }
        else {
            rebuildScaffold();
        }
        return 0;
    }

    void proceed(int n)   // proceedOptimization (main.cpp:109-118)
    {
        for (int i = 0; i < n && !converged && rc == OC_OK; ++i) {
            converged = solve1();
            if (iterNum >= cfg.maxNewtonIters) {
                converged = 1;
                rc = rc == OC_OK ? OC_ERR_NOT_CONVERGED : rc;
            }
        }
    }

    // ---- the dual step ------------------------------------------------
    double dualUpdate(double measure)   // updateLambda (main.cpp:614-618)
    {
        const double l = lam();
        const double x = std::max(0.0, measure - (upperBound - convTol / 2.0) + l / (1.0 - l));
        return x / (1.0 + x);
    }
    static double minChange(const std::vector<Cand>& L, double lambda)
    {
        double m = DBL_MAX;
        for (const Cand& c : L) {
            if (c.ec0 == DBL_MAX || c.ec1 == DBL_MAX) continue;
            m = std::min(m, c.ec0 * (1.0 - lambda) + c.ec1 * lambda);
        }
        return m;
    }
    // computeOptPicked (main.cpp:538-575): 1 when the second list's best is lower
    static int pickedSecond(const std::vector<Cand>& a, const std::vector<Cand>& b, double lambda)
    {
        return minChange(a, lambda) > minChange(b, lambda);
    }
    static int bestCand(const std::vector<Cand>& L, double lambda, double& change)   // main.cpp:577-595
    {
        change = DBL_MAX;
        int id = -1;
        for (int i = 0; i < (int)L.size(); ++i) {
            if (L[i].ec0 == DBL_MAX || L[i].ec1 == DBL_MAX) continue;
            const double c = L[i].ec0 * (1.0 - lambda) + L[i].ec1 * lambda;
            if (c < change) {
                change = c;
                id = i;
            }
        }
        return id;
    }
    static bool anyNegative(const std::vector<Cand>& L)   // checkCand (main.cpp:597-612)
    {
        for (const Cand& c : L)
            if (c.ec0 < 0.0 || c.ec1 < 0.0) return true;
        return false;
    }
    bool nearRecorded(double E_se, double lambda, double E_SD, double eps_E_se, double eps_lambda) const
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

    // updateLambda_stationaryV (main.cpp:620-884); false = stop the outer loop
    bool stationary(bool checkConvergence)
    {
        const double eps_E_se = 1.0e-3 * minEdgeLen() / virtualRadius;
        const double E_SD = energySD(), E_se = seam();
        const double measure = E_SD;
        const double eps_lambda = std::min(1.0e-3, std::abs(dualUpdate(measure) - lam()));
        if (iterNum != lastStationaryIterNum) {
            const double lambda = 1.0 - lam();
            const bool osc = nearRecorded(E_se, lambda, E_SD, eps_E_se, eps_lambda);
            if (measure <= upperBound && E_se < E_se_bestFeasible) {
                iterNum_bestFeasible = iterNum;
                bestFeasible = snapshot();
                E_se_bestFeasible = E_se;
            }
            if (osc && iterNum_bestFeasible >= 0) {
                if (iterNum_bestFeasible != iterNum) setConfig(bestFeasible);
                record(10);
                return false;
            }
            configs[E_se].emplace_back(lambda, E_SD);
        }
        lastStationaryIterNum = iterNum;
        if (checkConvergence && measure <= upperBound && measure >= upperBound - convTol) {
            if (iterNum_bestFeasible != iterNum && iterNum_bestFeasible >= 0) setConfig(bestFeasible);
            record(11);
            return false;
        }
        setLam(dualUpdate(measure));
        if (checkConvergence) {
            const std::vector<Cand>&B = lists[kBSplit], &I = lists[kISplit], &M = lists[kMerge];
            if (measure > upperBound) {
                if (!M.empty() && pickedSecond(B, M, 1.0 - lam()) == 1)
                    do {
                        setLam(dualUpdate(measure));
                    } while (pickedSecond(B, M, 1.0 - lam()) == 1 && rc == OC_OK);
                if (!anyNegative(I) && !anyNegative(B)) {
                    reQuery = true;   // filtering too strong
                }
                else {
                    double dB, dI;
                    int iB = bestCand(B, 1.0 - lam(), dB), iI = bestCand(I, 1.0 - lam(), dI);
                    while (dB > 0.0 && dI > 0.0 && rc == OC_OK) {
                        setLam(dualUpdate(measure));
                        iB = bestCand(B, 1.0 - lam(), dB);
                        iI = bestCand(I, 1.0 - lam(), dI);
                    }
                    if (dB <= 0.0) {
                        opType_queried = kBSplit;
                        queried = B[iB];
                    }
                    else {
                        opType_queried = kISplit;
                        queried = I[iI];
                    }
                }
            }
            else {
                bool noOp = true;
                for (const Cand& c : M)
                    if (c.ec0 != DBL_MAX) {
                        noOp = false;
                        break;
                    }
                if (noOp) {   // no merge left: end the process
                    setLam(1.0 - eps_lambda);
                    if (iterNum_bestFeasible != iterNum && iterNum_bestFeasible >= 0) setConfig(bestFeasible);
                    record(12);
                    return false;
                }
                if (pickedSecond(B, M, 1.0 - lam()) == 0)
                    do {
                        setLam(dualUpdate(measure));
                    } while (pickedSecond(B, M, 1.0 - lam()) == 0 && rc == OC_OK);
                double dM;
                int iM = bestCand(M, 1.0 - lam(), dM);
                while (dM > 0.0 && rc == OC_OK) {
                    setLam(dualUpdate(measure));
                    iM = bestCand(M, 1.0 - lam(), dM);
                }
                opType_queried = kMerge;
                queried = M[iM];
            }
        }
        if (lam() > 1.0 - eps_lambda) setLam(1.0 - eps_lambda);
        if (lam() < eps_lambda) setLam(eps_lambda);
        return true;
    }

    void finish()   // converge_preDrawFunc (main.cpp:886-911)
    {
        if (!cfg.bijective) {   // exact solve
            keep(oc_optimizer_set_allow_edec_rel_tol(opt, 0));
            converged = 0;
            propagate = 0;
            while (!converged && rc == OC_OK) proceed(1000);
        }
        finished = true;
    }

    // one pass of preDrawFunc in offline mode (main.cpp:913-1055)
    void step()
    {
        while (!converged && rc == OC_OK) proceed(1);
        if (rc != OC_OK) return;
        const double measure = energySD();
        if (converged == 2) {
            converged = 0;
            return;
        }
        // bijectivity on after a one-point initial cut: the scaffold starts
        // now (main.cpp:991-994); its energy enters at the next solve
        if (cfg.bijective && !scafOn()) {
            const auto t0 = std::chrono::steady_clock::now();
            keep(oc_optimizer_rebuild_scaffold(opt));
            ms[0] += ms_since(t0);
        }
        record(0);
        if (!stationary(false)) {
            finish();
            return;
        }
        if (createFracture(0.0, 0, cfg.topoLineSearch != 0)) {
            record(1);
            converged = 0;
            return;
        }
        if (rc != OC_OK) return;
        if (measure > upperBound && createFracture(0.0, 0, cfg.topoLineSearch != 0, true)) {
            record(2);
            converged = 0;
            return;
        }
        if (rc != OC_OK) return;
        if (!stationary(true)) {
            finish();
            return;
        }
        if (reQuery) {   // widen the interior-split filter until a split is taken
            auto widen = [&] {
                filterExp += std::log(2.0) / std::log((double)inSplitTotalAmt);
                filterExp = std::min(1.0, filterExp);
            };
            widen();
            int guard = 0;
            while (!createFracture(0.0, 0, cfg.topoLineSearch != 0, true) && rc == OC_OK && ++guard < 64) widen();
            reQuery = false;
            record(3);
        }
        else if (opType_queried >= 0) {
            createFracture(opType_queried, queried, cfg.topoLineSearch != 0);
            record(4 + opType_queried);
        }
        opType_queried = -1;
        converged = 0;
    }
};

extern "C" {

int oc_optcuts_default_config(oc_optcuts_config* c)
{
    if (!c) return OC_ERR_INVALID;
    c->upperBound = 4.1;
    c->bijective = 0;
    c->topoLineSearch = 1;
    c->filterExp = 0.6;
    c->topoOptions = 0;
    c->mlp = nullptr;
    c->topFrac = 0.1;
    c->maxNewtonIters = 100000;
    c->recordFeatures = 0;
    return OC_OK;
}

int oc_optcuts_create(oc_optimizer* opt, oc_mesh* mesh, const oc_optcuts_config* cfg, oc_optcuts** out)
{
    if (!opt || !mesh || !out) return OC_ERR_INVALID;
    oc_optcuts_config c;
    oc_optcuts_default_config(&c);
    if (cfg) c = *cfg;
    // b_d <= 4 is replaced by 4.1 (main.cpp:1266-1269)
    if (!(c.upperBound > 4.0)) c.upperBound = 4.1;
    if (!(c.filterExp > 0.0) || c.filterExp > 1.0 || c.maxNewtonIters <= 0) return OC_ERR_INVALID;
    oc_optcuts* o = new (std::nothrow) oc_optcuts;
    if (!o) return OC_ERR_NOMEM;
    o->opt = opt;
    o->mesh = mesh;
    o->cfg = c;
    o->upperBound = c.upperBound;
    o->filterExp = c.filterExp;
    double sc[3] = {0, 0, 0};
    oc_mesh_rest_constants(mesh, nullptr, sc);
    o->virtualRadius = sc[2] > 0.0 ? sc[2] : 1.0;
    oc_optimizer_get_iter_num(opt, &o->iterNum);
    int nC = 0;
    oc_mesh_get_topology(mesh, nullptr, nullptr, &nC, nullptr, nullptr, nullptr);
    std::vector<int> C(4 * (size_t)nC);
    if (nC) oc_mesh_get_topology(mesh, nullptr, nullptr, nullptr, nullptr, nullptr, C.data());
    o->initSeams.swap(C);
    *out = o;
    return OC_OK;
}

int oc_optcuts_mesh(const oc_optcuts* o, oc_mesh** mesh)
{
    if (!o || !mesh) return OC_ERR_INVALID;
    *mesh = o->mesh;
    return OC_OK;
}

int oc_optcuts_features(const oc_optcuts* o, int* nRows, float* X, float* target)
{
    if (!o || !nRows) return OC_ERR_INVALID;
    *nRows = static_cast<int>(o->featT.size());
    if (X) std::copy(o->featX.begin(), o->featX.end(), X);
    if (target) std::copy(o->featT.begin(), o->featT.end(), target);
    return OC_OK;
}

int oc_optcuts_initial_seams(const oc_optcuts* o, int* nRows, int* rows)
{
    if (!o || !nRows) return OC_ERR_INVALID;
    *nRows = static_cast<int>(o->initSeams.size() / 4);
    if (rows) std::copy(o->initSeams.begin(), o->initSeams.end(), rows);
    return OC_OK;
}

int oc_optcuts_destroy(oc_optcuts* o)
{
    delete o;
    return OC_OK;
}

int oc_optcuts_run(oc_optcuts* o, int maxSteps, int* finished)
{
    if (!o || maxSteps < 0) return OC_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < maxSteps && !o->finished && o->rc == OC_OK; ++s) o->step();
    o->ms[3] += ms_since(t0);
    if (finished) *finished = o->finished ? 1 : 0;
    return o->rc;
}

int oc_optcuts_state(oc_optcuts* o, double* out12)
{
    if (!o || !out12) return OC_ERR_INVALID;
    const double l = o->lam();
    const double sd = o->energySD(), se = o->seam();
    const double v[12] = {sd, se, 1.0 - l, l * sd + (1.0 - l) * se, (double)o->iterNum, (double)o->topoIter,
                          o->finished ? 1.0 : 0.0, (double)o->nVerts(), o->ms[0], o->ms[1], o->ms[2], o->ms[3]};
    std::copy(v, v + 12, out12);
    return OC_OK;
}

int oc_optcuts_events(const oc_optcuts* o, int* nRows, double* rows)
{
    if (!o || !nRows) return OC_ERR_INVALID;
    *nRows = static_cast<int>(o->events.size() / 6);
    if (rows) std::copy(o->events.begin(), o->events.end(), rows);
    return OC_OK;
}

int oc_optcuts_trace(const oc_optcuts* o, int* nRows, double* rows)
{
    if (!o || !nRows) return OC_ERR_INVALID;
    *nRows = static_cast<int>(o->trace.size() / 7);
    if (rows) std::copy(o->trace.begin(), o->trace.end(), rows);
    return OC_OK;
}

} // extern "C"
