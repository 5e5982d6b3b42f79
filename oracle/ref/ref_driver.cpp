// Headless driver for the reference OptCuts core, compiled from the
// reference's own sources (see oracle/ref/Makefile).  TEST INFRASTRUCTURE
// ONLY: it produces golden vectors and a CPU timing of the reference's own
// Newton loop; nothing in the product links or runs it.
//
// The reference's src/main.cpp cannot be compiled without an OpenGL viewer,
// so this file restates the part of it the hot path needs, with the viewer
// removed:
//   * the globals the core declares extern (src/Optimizer.cpp:28-33,
//     src/TriMesh.cpp:25-32; values as in src/main.cpp:38-80);
//   * the "no input UV" initialisation: per-component one-point cut or
//     cut_to_disk, boundary loop to circle, uniform-Laplacian harmonic map
//     (src/main.cpp:1379-1534);
//   * energyParams = {1 - lambda}, one SymDirichletEnergy, Optimizer
//     construction with scaffolding = bijective && !rand1PInitCut, and
//     precompute (src/main.cpp:1567-1574);
//   * the inner Newton loop solve(1) repeated (src/main.cpp:109-118, 917-921).
//
// Usage:
//   ref_driver <mesh.obj> <outdir/> <lambda> <newton_iters> [flags]
// flags: hess      dump per-triangle projected 6x6 Hessians at iteration 0
//        states    dump UV after every iteration
//        time      print wall-clock seconds per Newton iteration
//        nodump    write only the trace (for timing runs)
//        scaf      scaffolding on even after a one-point cut of a closed mesh
//        nobij     bijectivity off (the reference's bijectivity argument 0):
//                  no scaffold, local topology solves without air meshes
//        topo      after the Newton loop, run the topology queries the
//                  outer loop makes (TriMesh::querySplit boundary and
//                  interior, queryMerge) and dump their candidate lists
//                  (with bijectivity on, also the scaffold's air mesh the
//                  local air loops come from)
//        scafdump  dump, per iteration, the air mesh the iteration used
//                  (vertices, triangles, boundary map, fixed air vertices)
//                  and the augmented gradient / direction of iteration 0
//        outer     instead of <newton_iters> Newton iterations, the whole
//                  OptCuts run (src/main.cpp:913-1086, ref_outer.cpp) with
//                  b_d = 4.1 (bound=<b_d> to change it) for at most
//                  <newton_iters> outer passes; dumps the event record and
//                  the final state
// Outputs are .npy files in outdir (which must exist).

#include "Optimizer.hpp"
#include "SymDirichletEnergy.hpp"
#include "TriMesh.hpp"
#include "IglUtils.hpp"
#include "Timer.hpp"
#include "cut_to_disk.hpp"
#include "ref_outer.hpp"

#include <igl/readOBJ.h>
#include <igl/boundary_loop.h>
#include <igl/map_vertices_to_circle.h>
#include <igl/harmonic.h>
#include <igl/facet_components.h>
#include <igl/euler_characteristic.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <set>
#include <string>
#include <vector>

// ---- globals the reference core declares extern --------------------------
OptCuts::MethodType methodType = OptCuts::MT_OPTCUTS;
std::string outputFolderPath = "./";
bool fractureMode = false;
std::ofstream logFile;
Timer timer, timer_step;
std::vector<std::pair<double, double>> energyChanges_bSplit, energyChanges_iSplit, energyChanges_merge;
std::vector<std::vector<int>> paths_bSplit, paths_iSplit, paths_merge;
std::vector<Eigen::MatrixXd> newVertPoses_bSplit, newVertPoses_iSplit, newVertPoses_merge;
double filterExp_in = 0.6;
int inSplitTotalAmt;

// ---- tiny .npy writer -----------------------------------------------------
static void write_npy(const std::string& path, const void* data, const char* descr,
                      size_t elsize, const std::vector<size_t>& shape)
{
    std::string sh = "(";
    size_t n = 1;
    for (size_t i = 0; i < shape.size(); ++i) {
        sh += std::to_string(shape[i]);
        sh += (shape.size() == 1 || i + 1 < shape.size()) ? "," : "";
        if (i + 1 < shape.size()) sh += " ";
        n *= shape[i];
    }
    sh += ")";
    std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + sh + ", }";
    size_t total = 10 + hdr.size() + 1;
    size_t pad = (64 - total % 64) % 64;
    hdr += std::string(pad, ' ');
    hdr += '\n';
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    std::fwrite(magic, 1, 8, f);
    uint16_t hl = static_cast<uint16_t>(hdr.size());
    unsigned char hlb[2] = {static_cast<unsigned char>(hl & 0xff), static_cast<unsigned char>(hl >> 8)};
    std::fwrite(hlb, 1, 2, f);
    std::fwrite(hdr.data(), 1, hdr.size(), f);
    if (n) std::fwrite(data, elsize, n, f);
    std::fclose(f);
}

// Row-major copies of Eigen column-major matrices.
static void npy_mat(const std::string& path, const Eigen::MatrixXd& M)
{
    Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor> R = M;
    write_npy(path, R.data(), "<f8", 8, {static_cast<size_t>(M.rows()), static_cast<size_t>(M.cols())});
}
static void npy_mati(const std::string& path, const Eigen::MatrixXi& M)
{
    Eigen::Matrix<int, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor> R = M;
    write_npy(path, R.data(), "<i4", 4, {static_cast<size_t>(M.rows()), static_cast<size_t>(M.cols())});
}
static void npy_vec(const std::string& path, const Eigen::VectorXd& v)
{
    write_npy(path, v.data(), "<f8", 8, {static_cast<size_t>(v.size())});
}
static void npy_vecd(const std::string& path, const std::vector<double>& v)
{
    write_npy(path, v.data(), "<f8", 8, {v.size()});
}
static void npy_veci(const std::string& path, const std::vector<int>& v)
{
    write_npy(path, v.data(), "<i4", 4, {v.size()});
}

// Access to the Optimizer's protected iteration state (search direction,
// gradient, last energy) for golden dumps.
struct ProbeOptimizer : public OptCuts::Optimizer {
    using OptCuts::Optimizer::Optimizer;
    const Eigen::VectorXd& searchDirection() const { return searchDir; }
    const Eigen::VectorXd& grad() const { return gradient; }
    double targetG() const { return targetGRes; }
    double lastE() const { return lastEnergyVal; }
};

int main(int argc, char** argv)
{
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s mesh.obj outdir/ lambda iters [hess] [states] [time] [nodump]\n", argv[0]);
        return 1;
    }
    const std::string meshPath = argv[1];
    std::string out = argv[2];
    if (out.back() != '/') out += '/';
    const double lambda_init = std::stod(argv[3]);
    const int iters = std::stoi(argv[4]);
    bool dumpHess = false, dumpStates = false, doTime = false, noDump = false, forceScaf = false, scafDump = false;
    bool noBij = false, doTopo = false, doOuter = false;
    double bound = 4.1;
    for (int i = 5; i < argc; ++i) {
        if (!std::strcmp(argv[i], "hess")) dumpHess = true;
        else if (!std::strcmp(argv[i], "states")) dumpStates = true;
        else if (!std::strcmp(argv[i], "time")) doTime = true;
        else if (!std::strcmp(argv[i], "nodump")) noDump = true;
        else if (!std::strcmp(argv[i], "scaf")) forceScaf = true;
        else if (!std::strcmp(argv[i], "scafdump")) scafDump = true;
        else if (!std::strcmp(argv[i], "nobij")) noBij = true;
        else if (!std::strcmp(argv[i], "topo")) doTopo = true;
        else if (!std::strcmp(argv[i], "outer")) doOuter = true;
        else if (!std::strncmp(argv[i], "bound=", 6)) bound = std::stod(argv[i] + 6);
    }
    outputFolderPath = out;
    logFile.open(out + "log.txt");

    Eigen::MatrixXd V, UV, N;
    Eigen::MatrixXi F, FUV, FN;
    if (!igl::readOBJ(meshPath, V, UV, N, F, FUV, FN)) {
        std::fprintf(stderr, "cannot read %s\n", meshPath.c_str());
        return 1;
    }

    // ---- initial cut + Tutte embedding (src/main.cpp:1379-1534) ----------
    bool rand1PInitCut = false;
    Eigen::VectorXi C;
    igl::facet_components(F, C);
    const int n_components = C.maxCoeff() + 1;
    OptCuts::TriMesh temp(V, F, Eigen::MatrixXd(), Eigen::MatrixXi(), false);
    std::vector<Eigen::MatrixXi> F_component(n_components);
    std::vector<std::set<int>> V_ind_component(n_components);
    auto rebuild_components = [&]() {
        F_component.assign(n_components, Eigen::MatrixXi());
        V_ind_component.assign(n_components, std::set<int>());
        for (int triI = 0; triI < temp.F.rows(); ++triI) {
            F_component[C[triI]].conservativeResize(F_component[C[triI]].rows() + 1, 3);
            F_component[C[triI]].bottomRows(1) = temp.F.row(triI);
            for (int i = 0; i < 3; ++i) V_ind_component[C[triI]].insert(temp.F(triI, i));
        }
    };
    rebuild_components();
    while (true) {
        std::vector<int> to_cut;
        for (int ci = 0; ci < n_components; ++ci) {
            int EC = igl::euler_characteristic(temp.V, F_component[ci]) - temp.V.rows() + V_ind_component[ci].size();
            if (EC < 1) to_cut.emplace_back(-ci - 1);
            else if (EC == 2) to_cut.emplace_back(ci);
            else if (EC != 1) { std::fprintf(stderr, "unsupported component\n"); return 1; }
        }
        if (to_cut.empty()) break;
        for (auto ci : to_cut) {
            if (ci < 0) {
                ci = -ci - 1;
                std::vector<std::vector<int>> cuts;
                igl::cut_to_disk(F_component[ci], cuts);
                int cuts_made = 0;
                for (auto& seamI : cuts) {
                    if (seamI.front() == seamI.back()) {
                        cuts_made += temp.cutPath(std::vector<int>({seamI[seamI.size() - 3], seamI[seamI.size() - 2], seamI[seamI.size() - 1]}), true);
                        temp.initSeams = temp.cohE;
                        seamI.resize(seamI.size() - 2);
                    }
                    cuts_made += temp.cutPath(seamI, true);
                    temp.initSeams = temp.cohE;
                    if (cuts_made) break;
                }
                if (!cuts_made) { std::fprintf(stderr, "no cuts made\n"); return 1; }
            }
            else {
                temp.onePointCut(F_component[ci](0, 0));
                rand1PInitCut = (n_components == 1);
            }
        }
        rebuild_components();
    }
    int UVGridDim = 0;
    do { ++UVGridDim; } while (UVGridDim * UVGridDim < n_components);
    Eigen::VectorXi bnd_stacked;
    Eigen::MatrixXd bnd_uv_stacked;
    for (int ci = 0; ci < n_components; ++ci) {
        std::vector<std::vector<int>> bnd_all;
        igl::boundary_loop(F_component[ci], bnd_all);
        int longest = 0;
        for (int b = 1; b < (int)bnd_all.size(); ++b)
            if (bnd_all[longest].size() < bnd_all[b].size()) longest = b;
        bnd_stacked.conservativeResize(bnd_stacked.size() + bnd_all[longest].size());
        bnd_stacked.tail(bnd_all[longest].size()) = Eigen::VectorXi::Map(bnd_all[longest].data(), bnd_all[longest].size());
        Eigen::MatrixXd bnd_uv;
        igl::map_vertices_to_circle(temp.V_rest, bnd_stacked.tail(bnd_all[longest].size()), bnd_uv);
        double xOffset = ci % UVGridDim * 2.1, yOffset = ci / UVGridDim * 2.1;
        for (int r = 0; r < bnd_uv.rows(); ++r) { bnd_uv(r, 0) += xOffset; bnd_uv(r, 1) += yOffset; }
        bnd_uv_stacked.conservativeResize(bnd_uv_stacked.rows() + bnd_uv.rows(), 2);
        bnd_uv_stacked.bottomRows(bnd_uv.rows()) = bnd_uv;
    }
    Eigen::MatrixXd UV_Tutte;
    Eigen::SparseMatrix<double> A, M;
    OptCuts::IglUtils::computeUniformLaplacian(temp.F, A);
    igl::harmonic(A, M, bnd_stacked, bnd_uv_stacked, 1, UV_Tutte);
    OptCuts::TriMesh mesh(V, F, UV_Tutte, temp.F, false);

    const bool bijective = !noBij;
    std::vector<OptCuts::Energy*> energyTerms;
    std::vector<double> energyParams;
    energyParams.emplace_back(1.0 - lambda_init);
    energyTerms.emplace_back(new OptCuts::SymDirichletEnergy());
    const bool scaffolding = bijective && (!rand1PInitCut || forceScaf);

    // ---- initial-state dumps ---------------------------------------------
    if (!noDump) {
        npy_mat(out + "V_rest.npy", mesh.V_rest);
        npy_mat(out + "UV0.npy", mesh.V);
        npy_mati(out + "F.npy", mesh.F);
        npy_mati(out + "cohE.npy", mesh.cohE);
        npy_mati(out + "initSeams.npy", mesh.initSeams);
        npy_veci(out + "bnd.npy", std::vector<int>(bnd_stacked.data(), bnd_stacked.data() + bnd_stacked.size()));
        std::vector<int> fixed(mesh.fixedVert.begin(), mesh.fixedVert.end());
        npy_veci(out + "fixedVert.npy", fixed);
        Eigen::MatrixXd rest(mesh.F.rows(), 8);
        rest.col(0) = mesh.triArea; rest.col(1) = mesh.triAreaSq;
        rest.col(2) = mesh.e0SqLen; rest.col(3) = mesh.e1SqLen; rest.col(4) = mesh.e0dote1;
        rest.col(5) = mesh.e0SqLen_div_dbAreaSq; rest.col(6) = mesh.e1SqLen_div_dbAreaSq;
        rest.col(7) = mesh.e0dote1_div_dbAreaSq;
        npy_mat(out + "rest.npy", rest);
        double E_se;
        mesh.computeSeamSparsity(E_se, false);
        npy_vecd(out + "scalars.npy", {mesh.surfaceArea, mesh.avgEdgeLen, mesh.virtualRadius, E_se,
                                       lambda_init, scaffolding ? 1.0 : 0.0});
        // per-element energies, gradient, triplet Hessian of the initial state
        OptCuts::SymDirichletEnergy SD;
        Eigen::VectorXd e;
        SD.getEnergyValPerElem(mesh, e);
        npy_vec(out + "E_elem0.npy", e);
        double E0;
        SD.computeEnergyVal(mesh, E0);
        Eigen::VectorXd g;
        SD.computeGradient(mesh, g);
        npy_vec(out + "grad0.npy", g);
        if (dumpHess) {
            Eigen::VectorXd Hv; Eigen::VectorXi Hi, Hj;
            SD.computeHessian(mesh, &Hv, &Hi, &Hj);
            npy_vec(out + "H0_V.npy", Hv);
            npy_veci(out + "H0_I.npy", std::vector<int>(Hi.data(), Hi.data() + Hi.size()));
            npy_veci(out + "H0_J.npy", std::vector<int>(Hj.data(), Hj.data() + Hj.size()));
        }
    }

    ProbeOptimizer opt(mesh, energyTerms, energyParams, 0, false, scaffolding);
    auto t0 = std::chrono::steady_clock::now();
    opt.precompute();
    auto t1 = std::chrono::steady_clock::now();
    if (lambda_init > 0.0) fractureMode = true;

    if (doOuter) {
        RefOuterResult r = ref_outer_run(opt, energyParams, bound, bijective, rand1PInitCut, iters);
        const OptCuts::TriMesh& R = opt.getResult();
        write_npy(out + "outer_events.npy", r.events.data(), "<f8", 8, {r.events.size() / 6, 6});
        npy_vecd(out + "outer_final.npy", {r.E_SD, r.E_se, r.lambda, (double)r.iterNum, (double)r.topoIter,
                                           r.finished ? 1.0 : 0.0, r.seconds, bound});
        npy_mat(out + "outer_V.npy", R.V);
        npy_mati(out + "outer_F.npy", R.F);
        npy_mat(out + "outer_Vrest.npy", R.V_rest);
        npy_mati(out + "outer_cohE.npy", R.cohE);
        if (doTime)
            std::printf("outer loop: %s after %d Newton iterations, %d topology steps, %.2f s: E_SD %.9g E_se %.9g "
                        "lambda %.9g\n", r.finished ? "finished" : "stopped", r.iterNum, r.topoIter, r.seconds,
                        r.E_SD, r.E_se, r.lambda);
        return 0;
    }

    std::vector<double> trE, trESD, trG, trAlpha, trTime, trStatus, trEtot;
    trE.push_back(opt.getLastEnergyVal(true));
    trEtot.push_back(opt.getLastEnergyVal(false));
    std::vector<double> states;
    // per-iteration scaffolds, concatenated: air V rows, air F rows, bnd, fixed
    std::vector<double> scV;
    std::vector<int> scF, scB, scFix, scOff;   // scOff: per iteration nV, nF, nBnd, nFixed
    for (int it = 0; it < iters; ++it) {
        Eigen::MatrixXd Vprev = opt.getResult().V;
        if (scaffolding && scafDump) {
            const OptCuts::Scaffold& S = opt.getScaffold();
            Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor> AV = S.airMesh.V;
            Eigen::Matrix<int, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor> AF = S.airMesh.F;
            scV.insert(scV.end(), AV.data(), AV.data() + AV.size());
            scF.insert(scF.end(), AF.data(), AF.data() + AF.size());
            scB.insert(scB.end(), S.bnd.data(), S.bnd.data() + S.bnd.size());
            scFix.insert(scFix.end(), S.airMesh.fixedVert.begin(), S.airMesh.fixedVert.end());
            scOff.insert(scOff.end(), {(int)AV.rows(), (int)AF.rows(), (int)S.bnd.size(), (int)S.airMesh.fixedVert.size()});
        }
        auto s0 = std::chrono::steady_clock::now();
        int st = opt.solve(1);
        auto s1 = std::chrono::steady_clock::now();
        const Eigen::VectorXd& d = opt.searchDirection();
        const Eigen::MatrixXd& Vn = opt.getResult().V;
        double num = 0.0, den = 0.0;
        for (int v = 0; v < Vn.rows() && d.size() >= 2 * Vn.rows(); ++v) {
            for (int k = 0; k < 2; ++k) {
                num += (Vn(v, k) - Vprev(v, k)) * d[2 * v + k];
                den += d[2 * v + k] * d[2 * v + k];
            }
        }
        trE.push_back(opt.getLastEnergyVal(true));
        trEtot.push_back(opt.getLastEnergyVal(false));
        trESD.push_back(opt.getLastEnergyVal(true) / energyParams[0]);
        trG.push_back(opt.grad().squaredNorm());
        trAlpha.push_back(den > 0 ? num / den : 0.0);
        trTime.push_back(std::chrono::duration<double>(s1 - s0).count());
        trStatus.push_back(st);
        if (it == 0 && !noDump) npy_vec(out + "dir0.npy", d);
        if (it == 0 && !noDump && scaffolding) npy_vec(out + "gradw0.npy", opt.grad());
        if (dumpStates) {
            Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor> R = Vn;
            states.insert(states.end(), R.data(), R.data() + R.size());
        }
        if (doTime) std::printf("iter %d  %.6f s  E=%.17g  status=%d\n", it, trTime.back(), trE.back(), st);
        if (st == 1) break;
    }
    npy_vecd(out + "trace_E.npy", trE);
    npy_vecd(out + "trace_ESD.npy", trESD);
    npy_vecd(out + "trace_gsq.npy", trG);
    npy_vecd(out + "trace_alpha.npy", trAlpha);
    npy_vecd(out + "trace_time.npy", trTime);
    npy_vecd(out + "trace_status.npy", trStatus);
    npy_vecd(out + "trace_Etot.npy", trEtot);
    if (scaffolding && scafDump) {
        write_npy(out + "scaf_V.npy", scV.data(), "<f8", 8, {scV.size() / 2, 2});
        write_npy(out + "scaf_F.npy", scF.data(), "<i4", 4, {scF.size() / 3, 3});
        npy_veci(out + "scaf_bnd.npy", scB);
        npy_veci(out + "scaf_fixed.npy", scFix);
        write_npy(out + "scaf_off.npy", scOff.data(), "<i4", 4, {scOff.size() / 4, 4});
    }
    npy_vecd(out + "misc.npy", {std::chrono::duration<double>(t1 - t0).count(), opt.targetG()});
    if (dumpStates) {
        const size_t nv = opt.getResult().V.rows();
        write_npy(out + "UV_iters.npy", states.data(), "<f8", 8, {states.size() / (2 * nv), nv, 2});
    }
    if (doTopo) {
        // the topology queries of one outer iteration (main.cpp:1014-1020 ->
        // Optimizer::createFracture -> TriMesh::splitOrMerge / querySplit)
        OptCuts::TriMesh& R = opt.getResult();
        npy_mat(out + "topo_V.npy", R.V);
        npy_mati(out + "topo_F.npy", R.F);
        npy_mat(out + "topo_Vrest.npy", R.V_rest);
        npy_mati(out + "topo_cohE.npy", R.cohE);
        std::vector<int> fixedT(R.fixedVert.begin(), R.fixedVert.end());
        npy_veci(out + "topo_fixed.npy", fixedT);
        OptCuts::SymDirichletEnergy SD;
        Eigen::VectorXd dg;
        SD.computeDivGradPerVert(R, dg);
        npy_vec(out + "topo_divGrad.npy", dg);
        if (R.scaffold) {
            // bijectivity on: the air mesh the local air loops come from
            const OptCuts::Scaffold& sc = *R.scaffold;
            npy_mat(out + "topo_airV.npy", sc.airMesh.V);
            npy_mati(out + "topo_airF.npy", sc.airMesh.F);
            npy_veci(out + "topo_airBnd.npy", std::vector<int>(sc.bnd.data(), sc.bnd.data() + sc.bnd.size()));
        }
        const double lambda_t = 1.0 - energyParams[0];
        auto dump = [&](const std::string& tag, const std::vector<std::vector<int>>& paths,
                        const std::vector<Eigen::MatrixXd>& poses, const std::vector<std::pair<double, double>>& ec) {
            std::vector<int> pLen, pFlat, vRows;
            std::vector<double> vFlat, e;
            for (size_t c = 0; c < paths.size(); ++c) {
                pLen.push_back((int)paths[c].size());
                pFlat.insert(pFlat.end(), paths[c].begin(), paths[c].end());
                const Eigen::MatrixXd& P = c < poses.size() ? poses[c] : Eigen::MatrixXd();
                vRows.push_back((int)P.rows());
                for (int r = 0; r < P.rows(); ++r) { vFlat.push_back(P(r, 0)); vFlat.push_back(P(r, 1)); }
                e.push_back(c < ec.size() ? ec[c].first : 0.0);
                e.push_back(c < ec.size() ? ec[c].second : 0.0);
            }
            npy_veci(out + "topo_" + tag + "_pathLen.npy", pLen);
            npy_veci(out + "topo_" + tag + "_path.npy", pFlat);
            npy_veci(out + "topo_" + tag + "_posRows.npy", vRows);
            npy_vecd(out + "topo_" + tag + "_pos.npy", vFlat);
            npy_vecd(out + "topo_" + tag + "_energyChanges.npy", e);
        };
        double best[3];
        std::vector<int> bestPath, pathB, pathI;
        Eigen::MatrixXd bestPos, posB, posI;
        std::pair<double, double> bestEc;
        auto q0 = std::chrono::steady_clock::now();
        R.querySplit(lambda_t, false, false, best[0], pathB, posB, bestEc);
        auto q1 = std::chrono::steady_clock::now();
        dump("bSplit", paths_bSplit, newVertPoses_bSplit, energyChanges_bSplit);
        auto q2 = std::chrono::steady_clock::now();
        R.queryMerge(lambda_t, false, best[1], bestPath, bestPos, bestEc);
        auto q3 = std::chrono::steady_clock::now();
        dump("merge", paths_merge, newVertPoses_merge, energyChanges_merge);
        auto q4 = std::chrono::steady_clock::now();
        R.querySplit(lambda_t, false, true, best[2], pathI, posI, bestEc);
        auto q5 = std::chrono::steady_clock::now();
        dump("iSplit", paths_iSplit, newVertPoses_iSplit, energyChanges_iSplit);
        npy_vecd(out + "topo_best.npy", {best[0], best[1], best[2], lambda_t, (double)inSplitTotalAmt});
        const double tq[3] = {std::chrono::duration<double>(q1 - q0).count(),
                              std::chrono::duration<double>(q3 - q2).count(),
                              std::chrono::duration<double>(q5 - q4).count()};
        npy_vecd(out + "topo_seconds.npy", {tq[0], tq[1], tq[2]});
        if (doTime)
            std::printf("topology queries: boundary split %.3f s, merge %.3f s, interior split %.3f s\n", tq[0], tq[1],
                        tq[2]);
        // the operations themselves, applied to copies whatever their E_w
        // change (Optimizer::createFracture, Optimizer.cpp:373-440): the best
        // boundary split (then the merge query on that state and its best
        // merge) and the best interior split
        auto dumpState = [&](const std::string& tag, const OptCuts::TriMesh& M) {
            npy_mat(out + "topo_" + tag + "_V.npy", M.V);
            npy_mati(out + "topo_" + tag + "_F.npy", M.F);
            npy_mat(out + "topo_" + tag + "_Vrest.npy", M.V_rest);
            npy_mati(out + "topo_" + tag + "_cohE.npy", M.cohE);
        };
        npy_veci(out + "topo_opB_path.npy", pathB);
        npy_mat(out + "topo_opB_pos.npy", posB);
        npy_veci(out + "topo_opI_path.npy", pathI);
        npy_mat(out + "topo_opI_pos.npy", posI);
        if (best[0] > -1e300) {
            OptCuts::TriMesh Rb = R;
            Rb.splitEdgeOnBoundary(std::pair<int, int>(pathB[0], pathB[1]), posB);
            Rb.updateFeatures();
            dumpState("afterB", Rb);
            Rb.computeFeatures();   // as the next outer iteration sees it
            // with bijectivity on, the air mesh of the new state
            // (Optimizer::createFracture rebuilds the scaffold after every
            // operation, Optimizer.cpp:425-430)
            OptCuts::Scaffold scB;
            if (Rb.scaffold) {
                scB = OptCuts::Scaffold(Rb);
                Rb.scaffold = &scB;
                npy_mat(out + "topo_afterB_airV.npy", scB.airMesh.V);
                npy_mati(out + "topo_afterB_airF.npy", scB.airMesh.F);
                npy_veci(out + "topo_afterB_airBnd.npy",
                         std::vector<int>(scB.bnd.data(), scB.bnd.data() + scB.bnd.size()));
            }
            double bm;
            std::vector<int> pathM;
            Eigen::MatrixXd posM;
            Rb.queryMerge(lambda_t, false, bm, pathM, posM, bestEc);
            dump("mergeB", paths_merge, newVertPoses_merge, energyChanges_merge);
            npy_vecd(out + "topo_mergeB_best.npy", {bm});
            if (bm > -1e300) {
                npy_veci(out + "topo_opM_path.npy", pathM);
                npy_mat(out + "topo_opM_pos.npy", posM);
                Rb.mergeBoundaryEdges(std::pair<int, int>(pathM[0], pathM[1]), std::pair<int, int>(pathM[1], pathM[2]),
                                      posM.row(0));
                Rb.computeFeatures();
                dumpState("afterM", Rb);
            }
        }
        if (best[2] > -1e300) {
            OptCuts::TriMesh Ri = R;
            Ri.cutPath(pathI, true, 1, posI);
            dumpState("afterI", Ri);
        }
    }
    opt.flushEnergyFileOutput();
    opt.flushGradFileOutput();
    return 0;
}
