// GPU drop-in for the reference's OptCuts::Optimizer (src/Optimizer.hpp).
//
// This translation unit replaces src/Optimizer.cpp in a build of the
// reference: it defines the methods the reference's Optimizer.hpp declares,
// with the same signatures and return conventions, on top of the C ABI in
// include/optcuts_gpu.h.  main.cpp, TriMesh and Scaffold stay unchanged and
// link against it.  The Newton loop (gradient, PSD-projected Hessian,
// assembly, factorization, injective line search, scaffold) runs in the
// library; the topology queries of createFracture run batched on the device
// and fill the reference's energyChanges_* / paths_* / newVertPoses_* lists;
// every applied operation is mirrored onto the host TriMesh `result` with the
// reference's own TriMesh methods, so the caller sees the TriMesh it expects.
//
// Build: compile with the reference's include paths and -I<this repo>/include,
// link with liboc_gpu.so instead of Optimizer.o (oracle/ref/Makefile, target
// gpu-dropin, does exactly this for the headless reference driver).
#include "Optimizer.hpp"
#include "SymDirichletEnergy.hpp"
#include "Timer.hpp"

#include "optcuts_gpu.h"

#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <mutex>
#include <string>
#include <vector>

extern OptCuts::MethodType methodType;
extern const std::string outputFolderPath;
extern const bool fractureMode;
extern std::ofstream logFile;
extern Timer timer, timer_step;
extern std::vector<std::pair<double, double>> energyChanges_bSplit, energyChanges_iSplit, energyChanges_merge;
extern std::vector<std::vector<int>> paths_bSplit, paths_iSplit, paths_merge;
extern std::vector<Eigen::MatrixXd> newVertPoses_bSplit, newVertPoses_iSplit, newVertPoses_merge;
extern double filterExp_in;
extern int inSplitTotalAmt;

namespace {

using RowMatD = Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor>;
using RowMatI = Eigen::Matrix<int, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor>;

void check(int rc, const char* what)
{
    if (rc == OC_OK || rc == OC_ERR_NOT_CONVERGED) return;
    std::cerr << "GPU optimizer: " << what << " failed: " << oc_status_string(rc) << std::endl;
    std::exit(-1);   // the reference's fatal paths exit (Optimizer.cpp:65-67, 548-554)
}

// one context per process (device 0, its own stream)
oc_ctx* context()
{
    static std::once_flag once;
    static oc_ctx* ctx = nullptr;
    std::call_once(once, [] { check(oc_ctx_create(0, nullptr, &ctx), "oc_ctx_create"); });
    return ctx;
}

// device state of each Optimizer object (its header has no slot for it)
struct Device {
    oc_mesh* mesh = nullptr;
    oc_optimizer* opt = nullptr;
    bool lastPropagate = false;   // Optimizer::solve's static (Optimizer.cpp:205)
};
std::mutex g_mu;
std::map<const OptCuts::Optimizer*, Device> g_dev;

Device& dev(const OptCuts::Optimizer* o)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return g_dev[o];
}

void release(const OptCuts::Optimizer* o)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_dev.find(o);
    if (it == g_dev.end()) return;
    if (it->second.opt) oc_optimizer_destroy(it->second.opt);
    if (it->second.mesh) oc_mesh_destroy(it->second.mesh);
    g_dev.erase(it);
}

// the device mesh of a TriMesh (rest positions, UV, triangles, fixed
// vertices, cohesive edges)
oc_mesh* upload(const OptCuts::TriMesh& M)
{
    RowMatD vr = M.V_rest, uv = M.V;
    RowMatI F = M.F, C = M.cohE;
    std::vector<int> fixed(M.fixedVert.begin(), M.fixedVert.end());
    oc_mesh* m = nullptr;
    check(oc_mesh_create(context(), vr.data(), uv.data(), (int)M.V.rows(), F.data(), (int)F.rows(), fixed.data(),
                         (int)fixed.size(), 0.0, &m),
          "oc_mesh_create");
    check(oc_mesh_set_cohesive_edges(m, C.data(), (int)C.rows()), "oc_mesh_set_cohesive_edges");
    const int tails[3] = {M.curFracTail >= 0 && M.curFracTail < M.V.rows() ? M.curFracTail : -1,
                          M.curInteriorFracTails.first, M.curInteriorFracTails.second};
    oc_mesh_set_fracture_tails(m, tails);
    return m;
}

void download_uv(oc_mesh* m, OptCuts::TriMesh& M)
{
    RowMatD uv(M.V.rows(), 2);
    check(oc_mesh_get_uv(m, uv.data()), "oc_mesh_get_uv");
    M.V = uv;
}

struct Cand {
    double ew = -DBL_MAX, ec0 = 0.0, ec1 = 0.0;
    std::vector<int> path;
    Eigen::MatrixXd pos;
};

// one query result into the reference's candidate lists; returns the best
Cand read_list(const oc_topo_result* r, std::vector<std::pair<double, double>>* ec,
               std::vector<std::vector<int>>* paths, std::vector<Eigen::MatrixXd>* poses, int* pool)
{
    int n = 0, best = -1;
    oc_topo_result_info(r, &n, &best, pool, nullptr, nullptr, nullptr, nullptr);
    if (ec) {
        ec->assign(n, {0.0, 0.0});
        paths->assign(n, {});
        poses->assign(n, Eigen::MatrixXd());
    }
    Cand b;
    for (int c = 0; c < n; ++c) {
        int pl = 0, pr = 0;
        double e = 0.0, ch[2];
        oc_topo_result_candidate(r, c, &e, ch, nullptr, &pl, nullptr, &pr);
        std::vector<int> path(pl);
        RowMatD pos(pr, 2);
        oc_topo_result_candidate(r, c, nullptr, nullptr, path.data(), nullptr, pos.data(), nullptr);
        if (ec) {
            (*ec)[c] = {ch[0], ch[1]};
            (*paths)[c] = path;
            (*poses)[c] = pos;
        }
        if (c == best) {
            b.ew = e;
            b.ec0 = ch[0];
            b.ec1 = ch[1];
            b.path = path;
            b.pos = pos;
        }
    }
    return b;
}

// the operation on the host TriMesh with the reference's own methods, as
// Optimizer::createFracture / TriMesh::splitOrMerge apply it
void mirror(OptCuts::TriMesh& R, int op, const std::vector<int>& path, const Eigen::MatrixXd& pos)
{
    switch (op) {
    case 0:
        R.splitEdgeOnBoundary(std::pair<int, int>(path[0], path[1]), pos);
        R.updateFeatures();
        break;
    case 1:
        R.cutPath(path, true, 1, pos);
        R.fracTail.insert(path[0]);
        R.fracTail.insert(path[2]);
        R.curInteriorFracTails.first = path[0];
        R.curInteriorFracTails.second = path[2];
        R.curFracTail = -1;
        break;
    default:
        R.mergeBoundaryEdges(std::pair<int, int>(path[0], path[1]), std::pair<int, int>(path[1], path[2]), pos.row(0));
        R.computeFeatures();
        break;
    }
}

} // namespace

namespace OptCuts {

Optimizer::Optimizer(const TriMesh& p_data0, const std::vector<Energy*>& p_energyTerms,
                     const std::vector<double>& p_energyParams, int p_propagateFracture, bool p_mute,
                     bool p_scaffolding, const Eigen::MatrixXd& UV_bnds, const Eigen::MatrixXi& E,
                     const Eigen::VectorXi& bnd, bool p_useDense)
    : data0(p_data0), energyTerms(p_energyTerms), energyParams(p_energyParams)
{
    useDense = p_useDense;
    energyParamSum = 0.0;
    for (double p : energyParams) energyParamSum += p;
    gradient_ET.resize(energyTerms.size());
    energyVal_ET.resize(energyTerms.size());
    allowEDecRelTol = true;
    propagateFracture = p_propagateFracture;
    mute = p_mute;
    if (!mute) {
        file_energyValPerIter.open(outputFolderPath + "energyValPerIter.txt");
        file_gradientPerIter.open(outputFolderPath + "gradientPerIter.txt");
    }
    if (!data0.checkInversion()) std::exit(-1);
    globalIterNum = 0;
    relGL2Tol = 1.0e-12;
    topoIter = 0;
    needRefactorize = false;
    pardisoThreadAmt = 4;
    scaffolding = p_scaffolding;
    UV_bnds_scaffold = UV_bnds;
    E_scaffold = E;
    bnd_scaffold = bnd;
    w_scaf = energyParams[0] * 0.01;
    linSysSolver = nullptr;   // the Newton system lives on the device
    lastEnergyVal = lastEDec = targetGRes = 0.0;
    energyVal_scaffold = 0.0;
}

Optimizer::~Optimizer(void)
{
    if (file_energyValPerIter.is_open()) file_energyValPerIter.close();
    if (file_gradientPerIter.is_open()) file_gradientPerIter.close();
    release(this);
}

void Optimizer::precompute(void)
{
    result = data0;
    Device& d = dev(this);
    if (d.opt) oc_optimizer_destroy(d.opt);
    if (d.mesh) oc_mesh_destroy(d.mesh);
    d.mesh = upload(result);
    oc_optimizer_config cfg;
    oc_optimizer_default_config(&cfg);
    check(oc_optimizer_create(d.mesh, energyParams[0], &cfg, &d.opt), "oc_optimizer_create");
    check(oc_optimizer_set_rel_gl2_tol(d.opt, relGL2Tol), "setRelGL2Tol");
    if (scaffolding) check(oc_optimizer_rebuild_scaffold(d.opt), "Scaffold");
    check(oc_optimizer_precompute(d.opt), "precompute");
    lastEDec = 0.0;
    data_findExtrema = data0;
    updateTargetGRes();
    computeLastEnergyVal();
    if (!mute) {
        writeEnergyValToFile(true);
        std::cout << "E_initial = " << lastEnergyVal << std::endl;
    }
}

int Optimizer::solve(int maxIter)
{
    Device& d = dev(this);
    for (int iterI = 0; iterI < maxIter; ++iterI) {
        int res = 0;
        check(oc_optimizer_solve(d.opt, 1, &res), "solve");
        check(oc_optimizer_get_iter_num(d.opt, &globalIterNum), "getIterNum");
        check(oc_optimizer_last_edec(d.opt, &lastEDec), "lastEDec");
        download_uv(d.mesh, result);
        computeLastEnergyVal();
        if (!mute) writeEnergyValToFile(false);
        if (res == 1) return 1;
        if (propagateFracture > 0) {   // Optimizer.cpp:232-249
            if (!createFracture(lastEDec, propagateFracture)) {
                if (scaffolding) check(oc_optimizer_rebuild_scaffold(d.opt), "Scaffold");
                if (d.lastPropagate) {
                    d.lastPropagate = false;
                    return 2;
                }
            }
            else {
                d.lastPropagate = true;
            }
        }
        else if (scaffolding) {
            check(oc_optimizer_rebuild_scaffold(d.opt), "Scaffold");
        }
    }
    return 0;
}

void Optimizer::updatePrecondMtrAndFactorize(void) {}

void Optimizer::updateEnergyData(bool updateEVal, bool, bool)
{
    energyParamSum = 0.0;
    for (double p : energyParams) energyParamSum += p;
    updateTargetGRes();
    check(oc_optimizer_set_energy_param(dev(this).opt, energyParams[0]), "updateEnergyData");
    if (updateEVal) computeLastEnergyVal();
}

bool Optimizer::createFracture(int opType, const std::vector<int>& path, const Eigen::MatrixXd& newVertPos,
                               bool allowPropagate)
{
    ++topoIter;
    Device& d = dev(this);
    data_findExtrema = result;
    RowMatD pos = newVertPos;
    check(oc_optimizer_create_fracture(d.opt, opType, path.data(), (int)path.size(), pos.data(), (int)pos.rows()),
          "createFracture");
    mirror(result, opType, path, newVertPos);
    download_uv(d.mesh, result);
    computeLastEnergyVal();
    fractureInitiated = true;
    if (!mute) writeEnergyValToFile(false);
    if (allowPropagate) propagateFracture = 1 + (opType == 2);
    return true;
}

bool Optimizer::createFracture(double stressThres, int propType, bool allowPropagate, bool allowInSplit)
{
    if (propType == 0) ++topoIter;
    Device& d = dev(this);
    const double lambda_t = 1.0 - energyParams[0];
    data_findExtrema = result;
    Cand best;
    int op = -1;
    bool isMerge = false;
    if (propType == 0 && allowInSplit) {
        const int o = 1;
        oc_topo_result* r = nullptr;
        check(oc_topology_queries(d.mesh, &o, 1, lambda_t, filterExp_in, 0, nullptr, 0.1, &r), "querySplit");
        best = read_list(r, &energyChanges_iSplit, &paths_iSplit, &newVertPoses_iSplit, &inSplitTotalAmt);
        if (inSplitTotalAmt == 0) best.ew = 0.0;
        op = 1;
        oc_topo_result_destroy(r);
    }
    else if (propType == 0) {
        const int ops[2] = {0, 2};
        oc_topo_result* r[2] = {};
        check(oc_topology_queries(d.mesh, ops, 2, lambda_t, filterExp_in, 0, nullptr, 0.1, r), "splitOrMerge");
        int pool = 0;
        Cand s = read_list(r[0], &energyChanges_bSplit, &paths_bSplit, &newVertPoses_bSplit, &pool);
        if (pool == 0) s.ew = 0.0;
        Cand m = read_list(r[1], &energyChanges_merge, &paths_merge, &newVertPoses_merge, nullptr);
        if (m.ew > s.ew) {
            best = m;
            op = 2;
            isMerge = true;
        }
        else {
            best = s;
            op = 0;
        }
        oc_topo_result_destroy(r[0]);
        oc_topo_result_destroy(r[1]);
    }
    else {   // propagation at the fracture tail (TriMesh::splitEdge / mergeEdge)
        op = propType == 1 ? 0 : 2;
        isMerge = propType == 2;
        oc_topo_result* r = nullptr;
        check(oc_topology_query_tail(d.mesh, op, lambda_t, 0, &r), "query at the fracture tail");
        best = read_list(r, nullptr, nullptr, nullptr, nullptr);
        oc_topo_result_destroy(r);
    }
    if (!(best.ew > stressThres) || best.path.empty()) return false;
    RowMatD pos = best.pos;
    check(oc_optimizer_create_fracture(d.opt, op, best.path.data(), (int)best.path.size(), pos.data(), (int)pos.rows()),
          "createFracture");
    mirror(result, op, best.path, best.pos);
    download_uv(d.mesh, result);
    computeLastEnergyVal();
    fractureInitiated = true;
    if (!mute && propType == 0) writeEnergyValToFile(false);
    if (allowPropagate && propType == 0) propagateFracture = 1 + (isMerge ? 1 : 0);
    return true;
}

void Optimizer::setConfig(const TriMesh& config, int iterNum, int p_topoIter)
{
    topoIter = p_topoIter;
    globalIterNum = iterNum;
    result = config;
    RowMatD vr = result.V_rest, uv = result.V;
    RowMatI F = result.F, C = result.cohE;
    const int tails[3] = {result.curFracTail >= 0 && result.curFracTail < result.V.rows() ? result.curFracTail : -1,
                          result.curInteriorFracTails.first, result.curInteriorFracTails.second};
    check(oc_optimizer_set_state(dev(this).opt, (int)vr.rows(), vr.data(), uv.data(), (int)F.rows(), F.data(),
                                 (int)C.rows(), C.data(), tails, iterNum),
          "setConfig");
    updateEnergyData();
}

void Optimizer::setPropagateFracture(bool p_prop) { propagateFracture = p_prop; }

void Optimizer::setScaffolding(bool p_scaffolding)
{
    scaffolding = p_scaffolding;
    Device& d = dev(this);
    if (!d.opt) return;
    check(scaffolding ? oc_optimizer_rebuild_scaffold(d.opt) : oc_optimizer_clear_scaffold(d.opt), "setScaffolding");
}

void Optimizer::setUseDense(bool p_useDense) { useDense = p_useDense; }

void Optimizer::computeLastEnergyVal(void)
{
    Device& d = dev(this);
    if (!d.opt) return;
    check(oc_optimizer_get_last_energy(d.opt, &lastEnergyVal), "getLastEnergyVal");
    check(oc_optimizer_get_last_energy_scaffold(d.opt, &energyVal_scaffold), "getLastEnergyVal");
    energyVal_ET[0] = (lastEnergyVal - energyVal_scaffold) / energyParams[0];
}

void Optimizer::getGradientVisual(Eigen::MatrixXd& arrowVec) const { arrowVec.resize(0, 2); }
TriMesh& Optimizer::getResult(void) { return result; }
const Scaffold& Optimizer::getScaffold(void) const { return scaffold; }
const TriMesh& Optimizer::getAirMesh(void) const { return scaffold.airMesh; }
bool Optimizer::isScaffolding(void) const { return scaffolding; }
const TriMesh& Optimizer::getData_findExtrema(void) const { return data_findExtrema; }
int Optimizer::getIterNum(void) const { return globalIterNum; }
int Optimizer::getTopoIter(void) const { return topoIter; }

void Optimizer::setRelGL2Tol(double p_relTol)
{
    relGL2Tol = p_relTol;
    updateTargetGRes();
    Device& d = dev(this);
    if (d.opt) check(oc_optimizer_set_rel_gl2_tol(d.opt, relGL2Tol), "setRelGL2Tol");
}

void Optimizer::setAllowEDecRelTol(bool p_allowEDecRelTol)
{
    allowEDecRelTol = p_allowEDecRelTol;
    Device& d = dev(this);
    if (d.opt) check(oc_optimizer_set_allow_edec_rel_tol(d.opt, allowEDecRelTol ? 1 : 0), "setAllowEDecRelTol");
}

void Optimizer::flushEnergyFileOutput(void)
{
    file_energyValPerIter << buffer_energyValPerIter.str();
    file_energyValPerIter.flush();
    clearEnergyFileOutputBuffer();
}
void Optimizer::flushGradFileOutput(void)
{
    file_gradientPerIter << buffer_gradientPerIter.str();
    file_gradientPerIter.flush();
    clearGradFileOutputBuffer();
}
void Optimizer::clearEnergyFileOutputBuffer(void)
{
    buffer_energyValPerIter.str("");
    buffer_energyValPerIter.clear();
}
void Optimizer::clearGradFileOutputBuffer(void)
{
    buffer_gradientPerIter.str("");
    buffer_gradientPerIter.clear();
}

// the host-side pieces of the Newton iteration run in the library; these
// members keep their declarations' meaning for a caller that uses them
bool Optimizer::solve_oneStep(void) { return solve(1) == 1; }
bool Optimizer::lineSearch(void) { return false; }
void Optimizer::stepForward(const Eigen::MatrixXd&, const Eigen::MatrixXd&, TriMesh&, Scaffold&, double) const {}

void Optimizer::updateTargetGRes(void)
{
    targetGRes = energyParamSum * static_cast<double>(data0.V_rest.rows() - data0.fixedVert.size()) /
                 static_cast<double>(data0.V_rest.rows()) * relGL2Tol;
}

void Optimizer::computeEnergyVal(const TriMesh& data, const Scaffold&, double& energyVal, bool)
{
    energyTerms[0]->computeEnergyVal(data, energyVal_ET[0]);
    energyVal = energyParams[0] * energyVal_ET[0];
}

void Optimizer::computeGradient(const TriMesh& data, const Scaffold&, Eigen::VectorXd& g, bool)
{
    energyTerms[0]->computeGradient(data, gradient_ET[0]);
    g = energyParams[0] * gradient_ET[0];
}

void Optimizer::computeHessian(const TriMesh&, const Scaffold&) {}

void Optimizer::initStepSize(const TriMesh& data, double& stepSize) const
{
    for (Energy* e : energyTerms) e->initStepSize(data, searchDir, stepSize);
}

void Optimizer::writeEnergyValToFile(bool flush)   // Optimizer.cpp:706-728
{
    double E_se;
    result.computeSeamSparsity(E_se, !fractureMode);
    E_se /= result.virtualRadius;
    if (fractureMode) buffer_energyValPerIter << lastEnergyVal + (1.0 - energyParams[0]) * E_se;
    else buffer_energyValPerIter << lastEnergyVal;
    for (size_t eI = 0; eI < energyTerms.size(); ++eI) buffer_energyValPerIter << " " << energyVal_ET[eI];
    buffer_energyValPerIter << " " << E_se << " " << energyParams[0] << "\n";
    if (flush) flushEnergyFileOutput();
}

void Optimizer::writeGradL2NormToFile(bool flush)
{
    buffer_gradientPerIter << gradient.squaredNorm() << "\n";
    if (flush) flushGradFileOutput();
}

double Optimizer::getLastEnergyVal(bool excludeScaffold) const
{
    return (excludeScaffold && scaffolding) ? (lastEnergyVal - energyVal_scaffold) : lastEnergyVal;
}

} // namespace OptCuts
