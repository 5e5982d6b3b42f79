// Multifrontal sparse Cholesky on the device: the exact Newton solve behind
// LinSysSolver::analyze_pattern / factorize / solve
// (src/LinSysSolver/EigenLibSolver.cpp:71-107, SimplicialLDLT there).
#pragma once

#include "oc_internal.h"

#include <string>
#include <vector>

namespace oc {

constexpr int kTile = 32;      // dense tile edge (FP64) of the front kernels
constexpr int kRectRows = 32;  // rows of L21 per CTA in the forward GEMV (a warp's lanes)
constexpr int kRectCols = 8;   // columns of L21 per CTA in the backward GEMV^T (a warp each)
// levels whose fronts all have at most kNarrowK pivots use the narrow
// forward GEMV (a thread per row, kNarrowRows rows per CTA)
constexpr int kNarrowK = 64;
constexpr int kNarrowRows = 256;

// One node of the nested-dissection tree: its vertices (a separator, a
// leaf, or the forced root set) and its children (node indices; nodes are
// kept in postorder, children first).
struct NdNode {
    std::vector<int> S;
    std::vector<int> children;
};

struct TileTask {           // one CTA's work item in a tiled front kernel
    int front, i, j, p;
};

struct CholPlan {
    // ---- host symbolic data ----
    int nV = 0, nDof = 0, nFronts = 0, nLevels = 0;
    // the dissection tree the fronts come from (postorder; ndRoot: the
    // forced-root node, -1 without one), kept for incremental analyses;
    // fullFlops: the factor flops of the last full analysis, incremental:
    // incremental analyses since then
    std::vector<NdNode> nd;
    int ndRoot = -1;
    double fullFlops = 0.0;
    int incremental = 0;
    double ndMs = 0.0, symMs = 0.0;   // host time of the last analysis: dissection, front structures
    bool valid = true;                   // every index map resolved (checked before upload)
    std::vector<int> vertOrder;          // elimination order of vertices
    std::vector<int> permDof;            // permuted DOF -> original DOF
    std::vector<int> fk, fm, fparent, flevel, fdofStart;
    std::vector<long long> foff, fupd;   // front pool offset, update-vector offset
    std::vector<int> frowOff;            // offset into rowIdx (m entries per front)
    std::vector<int> rowIdx;             // permuted DOF of each front row
    std::vector<int> childOff, childList;            // children per front (CSR)
    std::vector<int> relOff;             // per front: offset into relIdx (m - k entries)
    std::vector<int> relIdx;             // child update row -> parent front row
    long long poolSize = 0, updSize = 0;
    double flops = 0.0;
    int maxM = 0;
    // per-level front lists and tiled task lists
    std::vector<int> levelFrontOff, levelFronts;
    // kind: 0 extend-add of child slot `child`, 1 panel solve, 5 trailing
    // update in 32 x 32 blocks (which also factors the next panel's diagonal
    // tile), 4 the first panel's diagonal tiles
    struct Launch { int kind; int level; int p; int taskOff; int taskCount; int child; };
    // factorization groups (subtrees and the chains that join them): group
    // g's launches launches[grpLaunchOff[g] .. grpLaunchOff[g+1]) run on
    // stream grpStream[g] (0 = the caller's stream), after the ends of groups
    // grpWait[grpWaitOff[g] .. grpWaitOff[g+1])
    static constexpr int kMaxFactStreams = 8, kMaxFactGroups = 2 * kMaxFactStreams;
    int factStreams = kMaxFactStreams;   // the most streams an analysis may use
    int nFactStreams = 1;                // streams the current plan uses
    std::vector<int> grpStream, grpWaitOff, grpWait, grpLaunchOff;
    std::vector<int> frontGroup;         // per front, its group
    std::vector<Launch> launches;        // in execution order
    std::vector<TileTask> tasks;
    // substitution work split: per level, (front, first row/column) chunks of
    // the rectangular part L21 (rows k..m) for the multi-CTA GEMV kernels
    std::vector<int> rectRowOff, rectColOff;   // nLevels + 1
    std::vector<int> levelMaxK, levelMaxM;     // per level: largest pivot count and front size
    std::vector<int2> rectRowTasks, rectColTasks;
    int2* dRectRowTasks = nullptr;
    int2* dRectColTasks = nullptr;
    double* tmpDot = nullptr;                  // nDof: L21^T x_B per pivot
    // assembly map from the block-CSR pattern
    std::vector<long long> asmDest;      // per slot: pool offset of entry (0,0) or -1
    std::vector<int> asmLd;              // per slot: leading dimension (front m)
    std::vector<unsigned char> asmDiag;  // per slot: diagonal block (lower half only)

    // ---- device memory kept across analyses (grown with headroom, freed by
    // chol_destroy): the index arrays at 256-byte-aligned offsets of one
    // buffer, the front pool, the update vectors, the three DOF vectors and
    // the two flags
    struct Keep {
        char* idx = nullptr;
        size_t idxCap = 0;
        double* pool = nullptr;
        size_t poolCap = 0;
        double* upd = nullptr;
        size_t updCap = 0;
        double* vec = nullptr;
        size_t vecCap = 0;
        int* flags = nullptr;
        cudaStream_t aux[kMaxFactStreams - 1] = {};   // factorization streams 1, 2, ..
        cudaEvent_t fork = nullptr, join[kMaxFactStreams - 1] = {}, grpEnd[kMaxFactGroups] = {};
    } keep;
    // ---- device copies (views into keep) ----
    double* pool = nullptr;
    double* upd = nullptr;
    double* yperm = nullptr;     // nDof
    double* xperm = nullptr;     // nDof
    int *dPermDof = nullptr, *dFk = nullptr, *dFm = nullptr, *dFdofStart = nullptr, *dFrowOff = nullptr;
    long long *dFoff = nullptr, *dFupd = nullptr;
    int *dRowIdx = nullptr, *dChildOff = nullptr, *dChildList = nullptr, *dRelOff = nullptr, *dRelIdx = nullptr;
    int* dLevelFronts = nullptr;
    TileTask* dTasks = nullptr;
    long long* dAsmDest = nullptr;
    int* dAsmLd = nullptr;
    unsigned char* dAsmDiag = nullptr;
    int* dFlag = nullptr;        // non-positive pivot count
    int* dSolveFlag = nullptr;   // set when a substitution's bounded wait ran out (sticky)
    bool onDevice = false;
    // captured launch sequences (fixed per topology)
    bool useGraphs = true;
    // largest thread-block cluster per front in the substitutions of the top
    // levels (1: one CTA per front everywhere); results are the same bits
    int solveCluster = 8;
    cudaGraphExec_t factGraph = nullptr, solveGraph = nullptr;
    const void* factKey = nullptr;
    const void* solveKey[2] = {nullptr, nullptr};
    double solveSign = 0.0;
};

// Symbolic analysis from a full-symmetric vertex block pattern (rowPtr/col
// over vertices incl. the diagonal).  Nested dissection by BFS level sets,
// or, given vertex coordinates xy (nV x 2), by geometric bisection at the
// median along the longer extent (for patterns whose few long edges -- a
// scaffold's air mesh around the UV domain -- would let BFS level sets wrap
// around the domain into long rings); rootVerts (optional) are kept out of
// the dissection and eliminated last, as one front above the dissection's
// roots.
void chol_analyze(CholPlan& P, int nV, const int* rowPtr, const int* col, int leafSize = 16,
                  const std::vector<int>* rootVerts = nullptr, const double* xy = nullptr);
// The front structures of a given dissection tree (nodes in postorder,
// rootNode the forced-root node or -1): everything chol_analyze does after
// its dissection.  P.valid is false when the tree does not separate the
// pattern (a child's update row missing from its parent front).
void chol_analyze_nodes(CholPlan& P, int nV, const int* rowPtr, const int* col, const std::vector<NdNode>& nodes,
                        int rootNode);
int chol_upload(CholPlan& P, std::string* err);
// drops the plan's device views and captured graphs (the kept device memory
// stays for the next upload)
void chol_free(CholPlan& P);
// chol_free, and the kept device memory released
void chol_destroy(CholPlan& P);
// Numeric factorisation of the block-CSR values (FP32 storage, FP64 fronts).
int chol_factorize(CholPlan& P, const DeviceBsr& b, cudaStream_t st, std::string* err, int* nBadPivots);
// Solves A x = sign * rhs.
int chol_solve(CholPlan& P, const double2* rhs, double2* x, double sign, cudaStream_t st, std::string* err);
// largest cluster per front in the substitutions (1..8; drops the captured
// solve graph so that the next solve records the new launches)
void chol_set_solve_cluster(CholPlan& P, int maxCluster);
// the most streams the factorization of the next analysis may use (1..8)
void chol_set_factor_streams(CholPlan& P, int streams);
// true when every front's children finish before it under the plan's
// streams and waits (same group at a lower level, an earlier group on the
// same stream, or a chain of waits), and the group tables are consistent
bool chol_groups_ordered(const CholPlan& P);
// tree levels whose pivot-part substitutions run as clusters, and the
// largest cluster size among them (1 when none)
int chol_solve_cluster_levels(const CholPlan& P, int* largest);
// whether a substitution kernel gave up a bounded wait since the upload
// (synchronises the stream)
int chol_solve_status(CholPlan& P, cudaStream_t st, int* timedOut);

} // namespace oc
