// Topology queries of the OptCuts outer loop (TriMesh::querySplit /
// queryMerge, src/TriMesh.cpp:548-951) with every candidate's local
// projected-Newton solve batched on the device (oc_fp64.cu, k_local_newton).
#pragma once

#include "oc_internal.h"

#include <memory>
#include <string>
#include <vector>

namespace oc {

enum { kOpBoundarySplit = 0, kOpInteriorSplit = 1, kOpMerge = 2 };

// One candidate as the reference records it in paths_* / newVertPoses_* /
// energyChanges_* (TriMesh.cpp:688-723, 916-930).
struct TopoCandidate {
    std::vector<int> path;      // bSplit: (vI, nbVI); iSplit: (p0, vI, p2); merge: 3-vertex zipper path
    std::vector<double> pos;    // newVertPos rows x 2
    double ec0 = 0.0, ec1 = 0.0;   // energyChanges (first, second)
    double EwDec = 0.0;         // E_w decrease used for the choice (interior splits halved)
};

// vertex adjacency and half-edges of one mesh topology, built once and
// shared by the queries of a topology step (opaque; oc_topo.cpp)
struct TopoAdjacency;
std::shared_ptr<TopoAdjacency> topo_adjacency(int nV, const int* F, int nF);

// device buffers, streams and events of the batched local solves, kept
// across queries (one per mesh; not for concurrent queries)
struct TopoWorkspace {
    void* buf[9] = {};
    size_t cap[9] = {};
    cudaStream_t aux[5] = {};
    cudaEvent_t ev[6] = {};
    unsigned long long uploaded = 0;    // batch whose problem arrays buf[1..5] hold
    unsigned long long nextBatch = 1;
    std::shared_ptr<void> host;         // per-thread scratch of the host problem assembly
    TopoWorkspace() = default;
    TopoWorkspace(const TopoWorkspace&) = delete;
    TopoWorkspace& operator=(const TopoWorkspace&) = delete;
    ~TopoWorkspace();
};

struct TopoQueryIn {
    int nV = 0, nF = 0;
    const int* F = nullptr;          // nF x 3
    const double* Vrest = nullptr;   // nV x 3
    const double* rest = nullptr;    // nF x 8 rest constants (triArea first)
    const double* UV = nullptr;      // nV x 2 (current)
    const int* cohE = nullptr;       // nCohE x 4
    int nCohE = 0;
    double surfaceArea = 0.0, avgEdgeLen = 0.0, virtualRadius = 0.0;
    const double* divGrad = nullptr; // nV (split filter)
    const DeviceMesh* dm = nullptr;  // device copy of the same mesh (rest constants, UV)
    const TopoAdjacency* adj = nullptr;   // adjacency of F (built here when null)
    int bigCluster = 0;              // largest cluster of blocks per local problem (0: the device's, 16 or 8)
    TopoWorkspace* ws = nullptr;     // reused device buffers (a temporary one when null)
    cudaStream_t st = nullptr;
    // fracture propagation (querySplit / queryMerge with propagate = true,
    // TriMesh.cpp:637-665, 828-833): the split candidates are exactly these
    // vertices (no filter), the merge candidates only the zipper-bottom pairs
    // forking at mergeFork (-1: none); mergeFork -2 = no restriction
    const int* candVerts = nullptr;
    int nCandVerts = 0;
    int mergeFork = -2;
    // candidate sharding across processes: only candidates c with
    // c % shardCount == shardRank are solved; the others keep EwDec -DBL_MAX
    // and energyChanges (DBL_MAX, DBL_MAX) (the list itself is the same on
    // every shard)
    int shardRank = 0, shardCount = 1;
    // bijective form (TriMesh::scaffold set): the whole-mesh air mesh the
    // local air loops come from (Scaffold::get1RingAirLoop /
    // getCornerAirLoop, Scaffold.cpp:339-520): nAirV x 2 positions (rows <
    // nAirBnd are the mesh vertices airBnd[i]), nAirF x 3 triangles
    // (counter-clockwise)
    bool bijective = false;
    const double* airV = nullptr;
    const int* airF = nullptr;
    const int* airBnd = nullptr;
    int nAirV = 0, nAirF = 0, nAirBnd = 0;
};

struct TopoStats {
    int nCandidates = 0, nProblems = 0, maxIters = 0, totalIters = 0, nonConverged = 0, nSelected = 0;
    long long totalTrials = 0;
    int airProblems = 0, airRejected = 0, airSteinerMax = 0, airCapped = 0;   // bijective form
    double buildMs = 0.0, solveMs = 0.0, probeMs = 0.0, exactMs = 0.0;
    // host phases of the whole step (shared by its operations): inputs
    // (positions, split filter, adjacency, air mesh copies), the air-loop
    // sources, ranking (features, MLP, selection), candidate lists
    double prepMs = 0.0, airMs = 0.0, rankMs = 0.0, finishMs = 0.0;
};

struct Mlp;
constexpr int kTopoNumFeatures = 32;
enum { kTopoFp32Hessian = 1, kTopoRecordFeatures = 2, kTopoLearned = 4, kTopoAutotune = 8, kTopoBijective = 16 };
// the autotuner's table: one row per (device, size class, count bucket,
// triangle bucket): the schedule it measured fastest and its milliseconds,
// next to the fixed rule's
struct ScheduleRecord {
    int device, cls, countBucket, triBucket;
    LocalSchedule best, rule;
    float bestMs, ruleMs;
    int candidates;
};
std::vector<ScheduleRecord> topo_schedule_table();
struct TopoOptions {
    int flags = 0;          // kTopoFp32Hessian | kTopoRecordFeatures | kTopoLearned
    Mlp* mlp = nullptr;     // learned proposal: ranks the local problems
    double topFrac = 0.1;   // fraction of them solved exactly
};
// per local problem: features (32), exact target (fraction of the local
// excess energy the solve removed; exhaustive queries), MLP prediction
// (learned queries); its candidate, its exact E_w decrease (NaN where not
// solved exactly) and the predicted one (learned queries), both on the
// candidate's scale (interior splits halved)
struct TopoExtras {
    std::vector<float> X, target, predicted;
    std::vector<int> cand;
    std::vector<double> ewExact, ewPred;
    // per problem: triangles, free vertices, Newton iterations, line-search
    // trials, SM cycles of the solve (the probe's for unselected problems)
    std::vector<int> nTri, nFree, iters, trials;
    std::vector<long long> cycles;
};

// opType: kOpBoundarySplit / kOpInteriorSplit (querySplit with
// splitInterior false / true) or kOpMerge (queryMerge).  filterExp is the
// interior-split filter exponent (filterExp_in, 0.6 by default).  best is
// the index of the largest EwDec (-1 when there is no candidate).
// opts.flags: kTopoFp32Hessian projects the local element Hessians in FP32
// (faster; energies, gradients, line search and local LDL^T stay FP64);
// kTopoRecordFeatures records every problem's features and exact target;
// kTopoLearned (with opts.mlp) solves only the MLP's top fraction exactly
int topo_query(const TopoQueryIn& in, int opType, double lambda_t, double filterExp, const TopoOptions& opts,
               std::vector<TopoCandidate>& out, int& best, int& candidatePool, TopoStats& stats, std::string* err,
               TopoExtras* extras = nullptr);

// One query's outputs (topo_query's, together)
struct TopoOpResult {
    std::vector<TopoCandidate> cands;
    int best = -1, pool = 0;
    TopoStats stats;
    TopoExtras extras;
};

// Several queries of one state at once (a topology step: boundary split,
// merge, interior split): their local problems built on host threads and
// solved in the same launches (probe and exact passes of the learned
// proposal shared), so the few large fans of one operation overlap the many
// small problems of another.  The result of each equals its topo_query.
int topo_query_ops(const TopoQueryIn& in, const int* ops, int nOps, double lambda_t, double filterExp,
                   const TopoOptions& opts, TopoOpResult* results, std::string* err);

// MLP inference on host rows (oc_mlp.cu)
int mlp_predict_host(Mlp& m, const float* X, int n, float* y);

// Applies one operation to host arrays (F nF x 3, Vrest nV x 3, UV nV x 2,
// cohE rows x 4) with the reference's vertex and cohesive-edge bookkeeping:
// boundary split TriMesh::splitEdgeOnBoundary (new vertices appended),
// interior split TriMesh::cutPath (one appended vertex, two cohesive rows),
// merge TriMesh::mergeBoundaryEdges (the merged copy removed by moving the
// last vertex into its slot).
// tails (optional, in/out): the fracture tails the reference keeps on the
// TriMesh -- curFracTail and curInteriorFracTails -- updated as
// splitEdgeOnBoundary (TriMesh.cpp:2891-2899), an interior split through
// createFracture / splitOrMerge (Optimizer.cpp:397-399, TriMesh.cpp:1039-1043)
// and mergeBoundaryEdges (TriMesh.cpp:3046-3048, 3169-3171) do.
// edit (optional, out): what happened to the vertex ids -- {0, src0, src1}:
// vertices appended, copies of src0 (and src1, -1 if none); {1, a, b}: b
// merged into a, then the last vertex moved into b's slot
int topo_apply(int opType, const int* path, int pathLen, const double* newVertPos, int posRows, std::vector<int>& F,
               std::vector<double>& Vrest, std::vector<double>& UV, std::vector<int>& cohE, std::string* err,
               int* tails = nullptr, int* edit = nullptr);

// igl::cut_to_disk as the reference vendors it (src/Utils/cut_to_disk.cpp):
// the cut graph of a genus >= 1 surface as vertex lists (a closed loop
// repeats its first vertex), host only
void topo_cut_to_disk(const int* F, int nF, std::vector<std::vector<int>>& cuts);

// TriMesh::cutPath(path, makeCoh = true) as the initial cutting uses it:
// boundary splits along the path (an interior path opened by the interior
// cut of its first three vertices), on host arrays; made: edges split
int topo_cut_path(const int* path, int pathLen, std::vector<int>& F, std::vector<double>& Vrest,
                  std::vector<double>& UV, std::vector<int>& cohE, int& made, std::string* err);

// the split filter alone (host): candidate vertices in the reference's order
int topo_split_candidates(int nV, const int* F, int nF, const double* divGrad, bool interior, double filterExp,
                          std::vector<int>& cands, int& pool);

} // namespace oc
