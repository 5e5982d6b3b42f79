// Host side of the C ABI (include/optcuts_gpu.h): context, device mesh,
// linear solver and the projected-Newton Optimizer, each mirroring the
// reference class it replaces (TriMesh, SymDirichletEnergy, LinSysSolver /
// EigenLibSolver, Optimizer).  No exception crosses the ABI; every entry
// point returns an oc_status.

#include "oc_airmesh.h"
#include "oc_chol.h"
#include "oc_internal.h"
#include "oc_mlp.h"
#include "oc_topo.h"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <array>
#include <new>
#include <numeric>
#include <string>
#include <vector>

struct oc_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    int nsm = 0;
    std::string err;
};

struct oc_optimizer;

struct oc_mesh {
    oc_ctx* ctx = nullptr;
    // the Optimizer whose scaffold is this mesh's (TriMesh::scaffold): the
    // air mesh the bijective topology queries take their local loops from
    oc_optimizer* scafOwner = nullptr;
    unsigned long long topoVersion = 0;   // advanced whenever F changes
    oc::DeviceMesh d;
    oc::Scratch scratch;
    std::vector<double> rest;       // nF x 8, TriMesh feature layout
    std::vector<double> Vrest;      // nV x 3
    std::vector<int> cohE;          // nCohE x 4 cohesive edge pairs (TriMesh::cohE)
    double* divGrad = nullptr;      // nV (lazy)
    double scalars[3] = {0, 0, 0};  // surfaceArea, avgEdgeLen, virtualRadius
    std::vector<int> F, fixed;
    double2* cornerBuf = nullptr;   // 3 x nF corner gradients
    double2* tmpV = nullptr;        // nV scratch
    double* hb = nullptr;           // 21 x nF packed Hessians
    double* tmpF = nullptr;         // nF x 36 scratch for API outputs (lazy)
    std::shared_ptr<oc::TopoAdjacency> adj;   // adjacency of F for topology queries (lazy)
    std::shared_ptr<oc::TopoWorkspace> topoWs;   // device buffers of the batched local solves (lazy)
    // fracture tails (TriMesh::curFracTail, curInteriorFracTails), kept by
    // the applied operations for fracture propagation
    int tails[3] = {-1, -1, -1};
    // the last topology operations' effect on the vertex ids, by the
    // topoVersion each produced: {version, kind, x, y, nV before} (kind 0:
    // copies of x (and y) appended; 1: y merged into x, the last vertex
    // moved into y's slot) -- what an incremental symbolic analysis needs
    std::vector<std::array<long long, 5>> editLog;
};

struct oc_linsys {
    oc_ctx* ctx = nullptr;
    oc::DeviceBsr b;
    oc::PcgWork wk;
    int nV = 0, nF = 0;
    std::vector<int> rowPtr, col, diagSlot;
    std::vector<unsigned char> rowFixed;
    int* dFlag = nullptr;
    double2 *tmpIn = nullptr, *tmpOut = nullptr;
    bool patternSet = false;
    int kind = OC_SOLVER_DIRECT;
    oc::CholPlan chol;
    // last set_pattern: host pattern + symbolic analysis, device allocation + upload (ms);
    // carryMs: the carried dissection tree it took (counted with the host part)
    double patternHostMs = 0.0, patternDevMs = 0.0, carryMs = 0.0;
    // the mesh state the plan was analysed for: its topoVersion, mesh
    // vertex count (the system's first vertices) and whether the plan's
    // root front is a scaffold clique
    unsigned long long analyzedVersion = ~0ULL;
    int analyzedMeshNV = 0;
};

struct oc_optimizer {
    oc_mesh* mesh = nullptr;
    oc_linsys* ls = nullptr;
    oc_optimizer_config cfg;
    double param = 1.0, relGL2Tol = 1e-12, targetGRes = 0.0;
    double lastEnergyVal = 0.0, lastEDec = 0.0;
    int globalIterNum = 0;
    bool precomputed = false;
    bool allowEDecRelTol = true;   // Optimizer::setAllowEDecRelTol (Optimizer.cpp:148-151)
    double2 *g = nullptr, *dir = nullptr, *uv0 = nullptr;
    // last-step diagnostics
    double lastStep = 0.0, lastRelRes = 0.0, lastGsq = 0.0;
    int lastPcgIters = 0, lastLsLaunches = 0;
    long long launches = 0;
    int badPivots = 0;
    cudaEvent_t ev[9] = {};
    double phaseMs[7] = {0, 0, 0, 0, 0, 0, 0};
    // last createFracture: mesh edit, device mesh, scaffold, pattern (host),
    // pattern (device), energy (ms)
    double applyMs[6] = {0, 0, 0, 0, 0, 0};
    // scaffold (the Optimizer's scaffolding branches): an air mesh over the
    // augmented vertex numbering [mesh vertices | air-only vertices]
    // (Scaffold::localVI2Global, Scaffold.cpp:179-184)
    int nV0 = 0, nFixed0 = 0;       // data0's vertex and fixed counts (targetGRes)
    bool scaf = false, patternStale = true, airContribStale = false, cliqueMode = false;
    oc::DeviceMesh air;
    // nWhole: system vertices incl. unused air slots (nV + capAir);
    // nWholeReal: nV + air-only vertices
    int nWhole = 0, nWholeReal = 0, capAir = 0, capWhole = 0, capAirF = 0, nAirV = 0, nBnd = 0;
    double wScaf = 0.0, airScale = 0.0, eScaf = 0.0;
    double2* wuv = nullptr;         // augmented UV (capWhole)
    double2* airCorner = nullptr;   // 3 x capAirF
    double* airHb = nullptr;        // 21 x capAirF
    std::vector<int> airFw, bnd;    // air triangles in augmented ids; boundary map
    std::vector<int> airF;          // air triangles in air-mesh ids
    // the mesh's boundary loops for the air-mesh rebuilds, kept while the
    // topology (the mesh's topoVersion) is the same
    std::vector<int> bndLoops, bndLoopStart, bndSeeds;
    unsigned long long bndVersion = ~0ULL;
};

namespace oc {
cudaStream_t ctx_stream(oc_ctx* ctx) { return ctx ? ctx->stream : nullptr; }
} // namespace oc

// milliseconds since t; t moves to now
static double ms_since(std::chrono::steady_clock::time_point& t)
{
    const auto n = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(n - t).count();
    t = n;
    return ms;
}

namespace {

int fail(oc_ctx* ctx, int code, const std::string& msg)
{
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_check(oc_ctx* ctx, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return OC_OK;
    return fail(ctx, OC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define OC_CUDA(ctx, call)                                   \
    do {                                                     \
        int _rc = cuda_check((ctx), (call), #call);          \
        if (_rc != OC_OK) return _rc;                        \
    } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t n)
{
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (n ? n : 1));
}

template <typename T>
cudaError_t upload(T* dst, const T* src, size_t n, cudaStream_t st)
{
    return cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, st);
}

// Reads s.result[0..n) to the host (synchronises the stream).
int read_result(oc_mesh* m, int n, double* out)
{
    OC_CUDA(m->ctx, cudaGetLastError());
    OC_CUDA(m->ctx, cudaMemcpyAsync(m->scratch.hostResult, m->scratch.result, sizeof(double) * n,
                                    cudaMemcpyDeviceToHost, m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    std::memcpy(out, m->scratch.hostResult, sizeof(double) * n);
    return OC_OK;
}

int read_min(oc_mesh* m, double* out)
{
    unsigned long long bits = 0;
    OC_CUDA(m->ctx, cudaGetLastError());
    OC_CUDA(m->ctx, cudaMemcpyAsync(m->scratch.hostResult, m->scratch.minBits, sizeof(bits), cudaMemcpyDeviceToHost,
                                    m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    std::memcpy(&bits, m->scratch.hostResult, sizeof(bits));
    std::memcpy(out, &bits, sizeof(bits));
    return OC_OK;
}

// TriMesh::computeFeatures rest constants (TriMesh.cpp:355-393), 8 per
// triangle: triArea, triAreaSq, e0SqLen, e1SqLen, e0dote1 and the three
// *_div_dbAreaSq values; triangles below areaThres take the degenerate-air
// clamp (:373-383).  Returns false on a zero-area triangle (:368-372).
bool rest_constants(const double* V_rest, const int* F, int nF, double areaThres, std::vector<double>& rest,
                    double& surfaceArea)
{
    rest.resize(8 * (size_t)nF);
    // per triangle on the host pool; the area is then summed in triangle
    // order, as the reference's loop does
    std::atomic<bool> invalid{false};
    oc::host_parallel_for(nF, 4096, [&](size_t t0, size_t t1) {
        for (size_t t = t0; t < t1; ++t) {
            const double* P1 = V_rest + 3 * (size_t)F[3 * t];
            const double* P2 = V_rest + 3 * (size_t)F[3 * t + 1];
            const double* P3 = V_rest + 3 * (size_t)F[3 * t + 2];
            const double a[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]};
            const double b[3] = {P3[0] - P1[0], P3[1] - P1[1], P3[2] - P1[2]};
            const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            double* r = &rest[8 * t];
            r[0] = 0.5 * std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            if (r[0] == 0.0) invalid = true;
            if (r[0] < areaThres) {
                r[0] = areaThres;
                r[1] = areaThres * areaThres;
                r[2] = r[3] = 4.0 / std::sqrt(3.0) * areaThres;
                r[4] = r[2] / 2.0;
                r[5] = r[6] = 2.0 / std::sqrt(3.0) / areaThres;
                r[7] = r[5] / 2.0;
            }
            else {
                r[1] = r[0] * r[0];
                r[2] = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
                r[3] = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
                r[4] = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
                r[5] = r[2] / 2. / r[1];
                r[6] = r[3] / 2. / r[1];
                r[7] = r[4] / 2. / r[1];
            }
        }
    });
    surfaceArea = 0.0;
    for (int t = 0; t < nF; ++t) surfaceArea += rest[8 * (size_t)t];   // the clamped area where clamped
    return !invalid;
}

void device_mesh_free(oc::DeviceMesh& d)
{
    cudaFree(d.F0); cudaFree(d.F1); cudaFree(d.F2);
    cudaFree(d.A2); cudaFree(d.w); cudaFree(d.e0); cudaFree(d.e1); cudaFree(d.e01);
    cudaFree(d.e0d); cudaFree(d.e1d); cudaFree(d.e01d); cudaFree(d.area);
    cudaFree(d.vcPtr); cudaFree(d.vcIdx); cudaFree(d.fixedMask);
    double2* uv = d.uv;
    d = oc::DeviceMesh{};
    d.uv = uv;   // owned by the caller
}

// Uploads a triangle set in the device layout (SoA indices and rest
// constants, vertex -> corner lists in triangle order, fixed mask); d.uv is
// left to the caller.  Frees what d held before.
int device_mesh_upload(oc_ctx* ctx, oc::DeviceMesh& d, int nV, const int* F, int nF, const std::vector<double>& rest,
                       double surfaceArea, const std::vector<unsigned char>& mask)
{
    // the arrays are reused while the mesh fits them (a scaffold's air mesh
    // is rebuilt every iteration with about the same size); otherwise they
    // are reallocated with some headroom
    const bool reuse = d.F0 && nF <= d.capF && nV <= d.capV;
    if (!reuse) device_mesh_free(d);
    d.nV = nV;
    d.nF = nF;
    std::vector<int> f0(nF), f1(nF), f2(nF);
    std::vector<double> col[9];
    for (auto& c : col) c.resize(nF);
    oc::host_parallel_for(nF, 8192, [&](size_t t0, size_t t1) {
        for (size_t t = t0; t < t1; ++t) {
            f0[t] = F[3 * t]; f1[t] = F[3 * t + 1]; f2[t] = F[3 * t + 2];
            const double* r = &rest[8 * t];
            col[0][t] = r[1];                    // triAreaSq
            col[1][t] = r[0] / surfaceArea;      // w (SymDirichletEnergy.cpp:41)
            col[2][t] = r[2]; col[3][t] = r[3]; col[4][t] = r[4];
            col[5][t] = r[5]; col[6][t] = r[6]; col[7][t] = r[7];
            col[8][t] = r[0];                    // triArea
        }
    });
    // vertex -> corners, sorted by triangle id
    std::vector<int> vcPtr(nV + 1, 0), vcIdx(3 * (size_t)nF);
    for (int t = 0; t < nF; ++t)
        for (int k = 0; k < 3; ++k) vcPtr[F[3 * t + k] + 1]++;
    for (int v = 0; v < nV; ++v) vcPtr[v + 1] += vcPtr[v];
    {
        std::vector<int> fill(vcPtr.begin(), vcPtr.end() - 1);
        for (int t = 0; t < nF; ++t)
            for (int k = 0; k < 3; ++k) vcIdx[fill[F[3 * t + k]]++] = k * nF + t;
    }
    cudaStream_t st = ctx->stream;
    int rc = OC_OK;
    auto chk = [&](cudaError_t e, const char* what) {
        if (rc == OC_OK && e != cudaSuccess) rc = fail(ctx, OC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    double** dcols[9] = {&d.A2, &d.w, &d.e0, &d.e1, &d.e01, &d.e0d, &d.e1d, &d.e01d, &d.area};
    if (!reuse) {
        const int capF = nF + nF / 4 + 64, capV = nV + nV / 16 + 64;
        chk(dalloc(&d.F0, capF), "alloc"); chk(dalloc(&d.F1, capF), "alloc"); chk(dalloc(&d.F2, capF), "alloc");
        for (int k = 0; k < 9; ++k) chk(dalloc(dcols[k], capF), "alloc");
        chk(dalloc(&d.vcPtr, capV + 1), "alloc");
        chk(dalloc(&d.vcIdx, 3 * (size_t)capF), "alloc");
        chk(dalloc(&d.fixedMask, capV), "alloc");
        if (rc == OC_OK) {
            d.capF = capF;
            d.capV = capV;
        }
    }
    if (rc == OC_OK) {
        chk(upload(d.F0, f0.data(), nF, st), "upload"); chk(upload(d.F1, f1.data(), nF, st), "upload");
        chk(upload(d.F2, f2.data(), nF, st), "upload");
        for (int k = 0; k < 9; ++k) chk(upload(*dcols[k], col[k].data(), nF, st), "upload");
        chk(upload(d.vcPtr, vcPtr.data(), nV + 1, st), "upload");
        chk(upload(d.vcIdx, vcIdx.data(), 3 * (size_t)nF, st), "upload");
        chk(upload(d.fixedMask, mask.data(), nV, st), "upload");
        chk(cudaStreamSynchronize(st), "sync");   // host staging vectors go out of scope
    }
    return rc;
}

// Full-symmetric 2x2-block pattern from the triangles (the vertex adjacency
// LinSysSolver::set_pattern reads from TriMesh::vNeighbor,
// LinSysSolver.hpp:37-135).  Fixed rows keep only their diagonal block.
// Also produces, per block slot, the ordered list of triangle contributions
// (t * 9 + a * 3 + b), free-free pairs only.  extraF adds adjacency only
// (air triangles, whose contributions are listed separately); clique adds
// every pair among its vertices.
void build_pattern(int nV, const int* F, int nF, const std::vector<unsigned char>& fixedMask,
                   std::vector<int>& rowPtr, std::vector<int>& col, std::vector<int>& diagSlot,
                   std::vector<int>& cPtr, std::vector<int>& cIdx, const int* extraF = nullptr, int nExtraF = 0,
                   const std::vector<int>* clique = nullptr, const int* nbPtr = nullptr, const int* nbIdx = nullptr)
{
    // candidate neighbours per row (counted, then filled), then each row
    // sorted and deduplicated on host threads and compacted
    std::vector<int> cnt(nV + 1, 0);
    auto count_tris = [&](const int* T, int n) {
        for (int t = 0; t < n; ++t)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    if (a != b && !fixedMask[T[3 * t + a]] && !fixedMask[T[3 * t + b]]) cnt[T[3 * t + a] + 1]++;
    };
    for (int v = 0; v < nV; ++v) cnt[v + 1] = 1;   // the diagonal
    count_tris(F, nF);
    if (extraF) count_tris(extraF, nExtraF);
    std::vector<int> cliqueFree;
    if (clique)
        for (int va : *clique)
            if (!fixedMask[va]) cliqueFree.push_back(va);
    for (int va : cliqueFree) cnt[va + 1] += static_cast<int>(cliqueFree.size()) - 1;
    // vertex neighbour lists (TriMesh::vNeighbor): both directions of each
    // listed pair between free vertices
    if (nbPtr)
        for (int va = 0; va < nV; ++va)
            for (int p = nbPtr[va]; p < nbPtr[va + 1]; ++p) {
                const int vb = nbIdx[p];
                if (vb != va && !fixedMask[va] && !fixedMask[vb]) {
                    cnt[va + 1]++;
                    cnt[vb + 1]++;
                }
            }
    for (int v = 0; v < nV; ++v) cnt[v + 1] += cnt[v];
    std::vector<int> raw(cnt[nV]);
    std::vector<int> fillPos(cnt.begin(), cnt.end() - 1);
    for (int v = 0; v < nV; ++v) raw[fillPos[v]++] = v;
    auto fill_tris = [&](const int* T, int n) {
        for (int t = 0; t < n; ++t)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    if (a == b) continue;
                    const int va = T[3 * t + a], vb = T[3 * t + b];
                    if (fixedMask[va] || fixedMask[vb]) continue;
                    raw[fillPos[va]++] = vb;
                }
    };
    fill_tris(F, nF);
    if (extraF) fill_tris(extraF, nExtraF);
    for (int va : cliqueFree)
        for (int vb : cliqueFree)
            if (vb != va) raw[fillPos[va]++] = vb;
    if (nbPtr)
        for (int va = 0; va < nV; ++va)
            for (int p = nbPtr[va]; p < nbPtr[va + 1]; ++p) {
                const int vb = nbIdx[p];
                if (vb != va && !fixedMask[va] && !fixedMask[vb]) {
                    raw[fillPos[va]++] = vb;
                    raw[fillPos[vb]++] = va;
                }
            }
    std::vector<int> uniq(nV);
    oc::host_parallel_for(nV, 4096, [&](size_t v0, size_t v1) {
        for (size_t v = v0; v < v1; ++v) {
            int* b = raw.data() + cnt[v];
            int* e = raw.data() + cnt[v + 1];
            std::sort(b, e);
            uniq[v] = static_cast<int>(std::unique(b, e) - b);
        }
    });
    rowPtr.assign(nV + 1, 0);
    for (int v = 0; v < nV; ++v) rowPtr[v + 1] = rowPtr[v] + uniq[v];
    col.resize(rowPtr[nV]);
    diagSlot.resize(nV);
    oc::host_parallel_for(nV, 4096, [&](size_t v0, size_t v1) {
        for (size_t v = v0; v < v1; ++v) {
            const int* b = raw.data() + cnt[v];
            std::copy(b, b + uniq[v], col.begin() + rowPtr[v]);
            diagSlot[v] = rowPtr[v] + static_cast<int>(std::lower_bound(b, b + uniq[v], (int)v) - b);
        }
    });
    std::vector<int>().swap(raw);
    const int nnzb = rowPtr[nV];
    std::vector<int> slotOf(9 * (size_t)nF, -1);
    oc::host_parallel_for(nF, 8192, [&](size_t t0, size_t t1) {
        for (size_t t = t0; t < t1; ++t)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    const int va = F[3 * t + a], vb = F[3 * t + b];
                    if (fixedMask[va] || fixedMask[vb]) continue;
                    const int* lo = col.data() + rowPtr[va];
                    const int* hi = col.data() + rowPtr[va + 1];
                    slotOf[9 * t + 3 * a + b] = static_cast<int>(std::lower_bound(lo, hi, vb) - col.data());
                }
    });
    cPtr.assign(nnzb + 1, 0);
    for (size_t k = 0; k < 9 * (size_t)nF; ++k)
        if (slotOf[k] >= 0) cPtr[slotOf[k] + 1]++;
    for (int s = 0; s < nnzb; ++s) cPtr[s + 1] += cPtr[s];
    cIdx.resize(cPtr[nnzb]);
    std::vector<int> fill(cPtr.begin(), cPtr.end() - 1);
    for (int t = 0; t < nF; ++t)        // increasing t: each list in triangle order
        for (int k = 0; k < 9; ++k) {
            const int s = slotOf[9 * (size_t)t + k];
            if (s >= 0) cIdx[fill[s]++] = 9 * t + k;
        }
}

// Per-slot contribution lists of the air triangles (augmented ids) in an
// existing pattern; false if a free-free pair has no slot.
bool air_contributions(const std::vector<int>& rowPtr, const std::vector<int>& col,
                       const std::vector<unsigned char>& fixedMask, const int* Fa, int nFa, std::vector<int>& aPtr,
                       std::vector<int>& aIdx)
{
    const int nV = static_cast<int>(rowPtr.size()) - 1;
    const int nnzb = rowPtr[nV];
    std::vector<int> slotOf(9 * (size_t)nFa, -1);
    aPtr.assign(nnzb + 1, 0);
    for (int t = 0; t < nFa; ++t)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int va = Fa[3 * t + a], vb = Fa[3 * t + b];
                if (fixedMask[va] || fixedMask[vb]) continue;
                const int* lo = col.data() + rowPtr[va];
                const int* hi = col.data() + rowPtr[va + 1];
                const int* f = std::lower_bound(lo, hi, vb);
                if (f == hi || *f != vb) return false;
                const int s = static_cast<int>(f - col.data());
                slotOf[9 * (size_t)t + 3 * a + b] = s;
                aPtr[s + 1]++;
            }
    for (int s = 0; s < nnzb; ++s) aPtr[s + 1] += aPtr[s];
    aIdx.resize(aPtr[nnzb] ? aPtr[nnzb] : 1);
    std::vector<int> fill(aPtr.begin(), aPtr.end() - 1);
    for (int t = 0; t < nFa; ++t)
        for (int k = 0; k < 9; ++k) {
            const int s = slotOf[9 * (size_t)t + k];
            if (s >= 0) aIdx[fill[s]++] = 9 * t + k;
        }
    return true;
}

void free_bsr(oc::DeviceBsr& b)
{
    cudaFree(b.rowPtr); cudaFree(b.col); cudaFree(b.val); cudaFree(b.diagSlot); cudaFree(b.rowFixed);
    cudaFree(b.cPtr); cudaFree(b.cIdx); cudaFree(b.dinv);
    cudaFree(b.aPtr); cudaFree(b.aIdx);
    b = oc::DeviceBsr{};
}

// mask: fixed rows for the pattern (diagonal only); rowFixed (optional):
// the fixed rows for the values where they differ (rows kept in the pattern
// but assembled as fixed, e.g. the padding slots of a scaffold clique)
// The dissection tree of the plan last analysed, carried through the
// topology operations applied since (edits: {version, kind, x, y, nV
// before}, in order): a copy joins its source vertex's node, a merged
// vertex the lowest common ancestor of the two nodes (a node above both
// separates everything they did), the last vertex moved into a removed
// slot keeps its node; system vertices past the mesh's (the scaffold's air
// slots) and the clique (scaffold boundary and air) go to the root node,
// which every other node descends from; nodes left empty are spliced out.
// Every separator of the old tree still separates the new pattern, so the
// front structures follow without a new dissection.  False when the tree
// cannot be carried (no root where a clique now needs one, two merged
// vertices in different trees).
bool carry_dissection(const oc::CholPlan& P, int oldMeshNV, const std::vector<std::array<long long, 5>>& edits,
                      int newMeshNV, int nSys, const std::vector<int>* clique, std::vector<oc::NdNode>& out,
                      int& rootNode)
{
    const int nOld = static_cast<int>(P.nd.size());
    if (nOld == 0 || (clique != nullptr) != (P.ndRoot >= 0)) return false;
    std::vector<int> parent(nOld, -1);
    for (int f = 0; f < nOld; ++f)
        for (int c : P.nd[f].children) parent[c] = f;
    std::vector<int> nodeOf(P.nV, -1);
    std::vector<long long> key(P.nV, 0);
    long long k = 0;
    for (int f = 0; f < nOld; ++f)
        for (int v : P.nd[f].S) {
            if (v < 0 || v >= P.nV) return false;
            nodeOf[v] = f;
            key[v] = k++;
        }
    if (oldMeshNV > P.nV) return false;
    std::vector<int> mn(nodeOf.begin(), nodeOf.begin() + oldMeshNV);
    std::vector<long long> mk(key.begin(), key.begin() + oldMeshNV);
    const int root = P.ndRoot;
    auto lca = [&](int x, int y) {
        for (int guard = 0; x != y && guard <= 2 * nOld; ++guard) {
            if (x < 0 || y < 0) return -1;
            if (x < y) x = parent[x];
            else y = parent[y];
        }
        return x == y ? x : -1;
    };
    for (const auto& e : edits) {
        const int n = static_cast<int>(mn.size());
        if (e[4] != n) return false;
        if (e[1] == 0) {
            for (int j = 2; j <= 3; ++j) {
                const long long src = e[j];
                if (src < 0) continue;
                if (src >= n) return false;
                mn.push_back(mn[src]);
                mk.push_back(k++);
            }
        }
        else {
            const long long a = e[2], b = e[3];
            if (a < 0 || b < 0 || a >= n || b >= n) return false;
            const int na = mn[a], nb = mn[b];
            int m = (na == root || nb == root) ? root : lca(na, nb);
            if (m < 0) return false;
            mn[a] = m;
            const int back = n - 1;
            if (b < back) {
                mn[b] = mn[back];
                mk[b] = mk[back];
            }
            mn.pop_back();
            mk.pop_back();
        }
    }
    if (static_cast<int>(mn.size()) != newMeshNV || nSys < newMeshNV) return false;
    std::vector<int> node(nSys, root);
    std::vector<long long> vkey(nSys, 0);
    for (int v = 0; v < newMeshNV; ++v) {
        node[v] = mn[v];
        vkey[v] = mk[v];
    }
    for (int v = newMeshNV; v < nSys; ++v) vkey[v] = k++;
    std::vector<char> inClique(nSys, 0);
    if (clique)
        for (int v : *clique) {
            if (v < 0 || v >= nSys) return false;
            node[v] = root;
            inClique[v] = 1;
        }
    for (int v = 0; v < nSys; ++v)
        if (node[v] < 0) return false;
    // vertices per node, in their old elimination order (the root: the
    // clique's order, then the vertices that stayed there)
    std::vector<std::vector<int>> S(nOld);
    // the keys are distinct and below k: the order by key is a bucket fill
    std::vector<int> byKey(static_cast<size_t>(k), -1);
    for (int v = 0; v < nSys; ++v) {
        if (vkey[v] < 0 || vkey[v] >= k || byKey[vkey[v]] >= 0) return false;
        byKey[vkey[v]] = v;
    }
    for (int v : byKey)
        if (v >= 0 && !inClique[v]) S[node[v]].push_back(v);
    if (clique) {
        std::vector<int> rs(clique->begin(), clique->end());
        rs.insert(rs.end(), S[root].begin(), S[root].end());
        S[root].swap(rs);
    }
    // splice out empty nodes (not the root); renumber in postorder
    std::vector<int> newIdx(nOld, -1);
    int nNew = 0;
    for (int f = 0; f < nOld; ++f)
        if (!S[f].empty() || f == root) newIdx[f] = nNew++;
    auto keptParent = [&](int f) {
        int p = parent[f];
        while (p >= 0 && newIdx[p] < 0) p = parent[p];
        return p;
    };
    out.assign(nNew, oc::NdNode{});
    for (int f = 0; f < nOld; ++f) {
        if (newIdx[f] < 0) continue;
        out[newIdx[f]].S.swap(S[f]);
        const int p = keptParent(f);
        if (p >= 0) out[newIdx[p]].children.push_back(newIdx[f]);
    }
    rootNode = root >= 0 ? newIdx[root] : -1;
    return true;
}

int linsys_set_pattern(oc_linsys* ls, int nV, const int* F, int nF, const std::vector<unsigned char>& mask,
                       const int* extraF = nullptr, int nExtraF = 0, const std::vector<int>* clique = nullptr,
                       const double* xy = nullptr, const std::vector<unsigned char>* rowFixed = nullptr,
                       const int* nbPtr = nullptr, const int* nbIdx = nullptr,
                       const std::vector<oc::NdNode>* carried = nullptr, int carriedRoot = -1,
                       const std::vector<int>* rootVerts = nullptr)
{
    oc_ctx* ctx = ls->ctx;
    auto t = std::chrono::steady_clock::now();
    std::vector<int> cPtr, cIdx;
    build_pattern(nV, F, nF, mask, ls->rowPtr, ls->col, ls->diagSlot, cPtr, cIdx, extraF, nExtraF, clique, nbPtr,
                  nbIdx);
    ls->patternHostMs = ms_since(t) + ls->carryMs;
    ls->carryMs = 0.0;
    ls->patternDevMs = 0.0;
    ls->rowFixed = rowFixed ? *rowFixed : mask;
    free_bsr(ls->b);
    oc::pcg_free(ls->wk);
    cudaFree(ls->tmpIn); cudaFree(ls->tmpOut);
    ls->tmpIn = ls->tmpOut = nullptr;
    oc::DeviceBsr& b = ls->b;
    b.nRows = nV;
    b.nnzb = ls->rowPtr[nV];
    cudaStream_t st = ctx->stream;
    OC_CUDA(ctx, dalloc(&b.rowPtr, nV + 1));
    OC_CUDA(ctx, dalloc(&b.col, b.nnzb));
    OC_CUDA(ctx, dalloc(&b.val, b.nnzb));
    OC_CUDA(ctx, dalloc(&b.diagSlot, nV));
    OC_CUDA(ctx, dalloc(&b.rowFixed, nV));
    OC_CUDA(ctx, dalloc(&b.cPtr, cPtr.size()));
    OC_CUDA(ctx, dalloc(&b.cIdx, cIdx.size()));
    OC_CUDA(ctx, dalloc(&b.dinv, nV));
    OC_CUDA(ctx, upload(b.rowPtr, ls->rowPtr.data(), nV + 1, st));
    OC_CUDA(ctx, upload(b.col, ls->col.data(), b.nnzb, st));
    OC_CUDA(ctx, upload(b.diagSlot, ls->diagSlot.data(), nV, st));
    OC_CUDA(ctx, upload(b.rowFixed, ls->rowFixed.data(), nV, st));
    OC_CUDA(ctx, upload(b.cPtr, cPtr.data(), cPtr.size(), st));
    OC_CUDA(ctx, upload(b.cIdx, cIdx.data(), cIdx.size(), st));
    OC_CUDA(ctx, cudaMemsetAsync(b.val, 0, sizeof(oc::Blk2) * (size_t)(b.nnzb ? b.nnzb : 1), st));
    oc::pcg_alloc(ls->wk, nV, ctx->device);
    OC_CUDA(ctx, cudaGetLastError());
    OC_CUDA(ctx, dalloc(&ls->tmpIn, nV));
    OC_CUDA(ctx, dalloc(&ls->tmpOut, nV));
    if (!ls->dFlag) OC_CUDA(ctx, dalloc(&ls->dFlag, 4));
    OC_CUDA(ctx, cudaStreamSynchronize(st));   // host vectors above go out of scope
    ls->nV = nV;
    ls->nF = nF;
    ls->patternSet = true;
    oc::chol_free(ls->chol);
    if (ls->kind == OC_SOLVER_DIRECT) {
        // analyze_pattern (EigenLibSolver.cpp:71-77): symbolic factorisation;
        // a clique (scaffold boundary + air vertices) is eliminated last
        ls->patternDevMs += ms_since(t);
        bool done = false;
        if (carried) {
            // the carried dissection tree: front structures only; a full
            // analysis when it does not separate the pattern, after 64
            // carried analyses, or once the factor cost grew 30% over the
            // last full analysis's
            const double full = ls->chol.fullFlops;
            if (ls->chol.incremental < 64 && full > 0.0) {
                ++ls->chol.incremental;
                ls->chol.ndMs = 0.0;
                oc::chol_analyze_nodes(ls->chol, nV, ls->rowPtr.data(), ls->col.data(), *carried, carriedRoot);
                ls->chol.nd = *carried;
                done = ls->chol.valid && ls->chol.flops <= 1.3 * full;
            }
        }
        // a clique, or the given root set, is eliminated last as one front
        if (!done) oc::chol_analyze(ls->chol, nV, ls->rowPtr.data(), ls->col.data(), 16, rootVerts ? rootVerts : clique, xy);
        ls->patternHostMs += ms_since(t);
        std::string err;
        int rc = oc::chol_upload(ls->chol, &err);
        if (rc) return fail(ctx, rc, err);
    }
    ls->patternDevMs += ms_since(t);
    return OC_OK;
}

// numeric factorisation (direct) or preconditioner (PCG); fixedDiag > 0 sets
// the fixed rows' diagonal blocks to fixedDiag * I first
int linsys_factor(oc_linsys* ls, double fixedDiag, int* nBad, double fixedDiag2 = 0.0)
{
    oc_ctx* ctx = ls->ctx;
    cudaStream_t st = ctx->stream;
    OC_CUDA(ctx, cudaMemsetAsync(ls->dFlag, 0, sizeof(int), st));
    if (fixedDiag > 0.0) oc::launch_precond_fixed(ls->b, fixedDiag, st, ls->dFlag, fixedDiag2);
    else oc::launch_precond(ls->b, st, ls->dFlag);
    int bad = 0;
    if (ls->kind == OC_SOLVER_DIRECT) {
        std::string err;
        int rc = oc::chol_factorize(ls->chol, ls->b, st, &err, &bad);
        if (rc) return fail(ctx, rc, err);
    }
    else {
        OC_CUDA(ctx, cudaMemcpyAsync(&bad, ls->dFlag, sizeof(int), cudaMemcpyDeviceToHost, st));
        OC_CUDA(ctx, cudaStreamSynchronize(st));
    }
    if (nBad) *nBad = bad;
    return OC_OK;
}

void record(oc_optimizer* o, int k)
{
    if (o->cfg.timing) cudaEventRecord(o->ev[k], o->mesh->ctx->stream);
}

} // namespace

extern "C" {

const char* oc_status_string(int s)
{
    switch (s) {
    case OC_OK: return "ok";
    case OC_ERR_INVALID: return "invalid argument";
    case OC_ERR_INVERTED: return "inverted triangle";
    case OC_ERR_NOT_CONVERGED: return "PCG did not converge";
    case OC_ERR_TIMEOUT: return "device loop budget exceeded";
    case OC_ERR_BOUNDS: return "index out of bounds";
    case OC_ERR_CUDA: return "CUDA error";
    case OC_ERR_DEGENERATE: return "zero-area rest triangle";
    case OC_ERR_NOT_SPD: return "non-positive diagonal block";
    case OC_ERR_NOMEM: return "out of memory";
    default: return "unknown status";
    }
}

int oc_ctx_create(int device, void* stream, oc_ctx** out)
{
    if (!out) return OC_ERR_INVALID;
    *out = nullptr;
    oc_ctx* c = new (std::nothrow) oc_ctx;
    if (!c) return OC_ERR_NOMEM;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) {
        if (stream) {
            c->stream = static_cast<cudaStream_t>(stream);
        }
        else {
            e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
            c->ownStream = true;
        }
    }
    if (e != cudaSuccess) {
        delete c;
        return OC_ERR_CUDA;
    }
    *out = c;
    return OC_OK;
}

int oc_ctx_destroy(oc_ctx* c)
{
    if (!c) return OC_ERR_INVALID;
    if (c->ownStream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return OC_OK;
}

const char* oc_last_error(const oc_ctx* c) { return c ? c->err.c_str() : "null context"; }

int oc_ctx_synchronize(oc_ctx* c)
{
    if (!c) return OC_ERR_INVALID;
    OC_CUDA(c, cudaStreamSynchronize(c->stream));
    return OC_OK;
}

// ------------------------------------------------------------------ mesh
int oc_mesh_create(oc_ctx* ctx, const double* V_rest, const double* UV, int nV, const int* F, int nF,
                   const int* fixedVert, int nFixed, double areaThres, oc_mesh** out)
{
    if (!ctx || !out || !V_rest || !UV || !F || nV <= 0 || nF <= 0 || nFixed < 0 || (nFixed && !fixedVert))
        return fail(ctx, OC_ERR_INVALID, "oc_mesh_create: bad arguments");
    if ((long long)nF * 9 >= (1LL << 31)) return fail(ctx, OC_ERR_INVALID, "oc_mesh_create: too many triangles");
    *out = nullptr;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return fail(ctx, OC_ERR_INVALID, "oc_mesh_create: vertex index out of range");
    for (int i = 0; i < nFixed; ++i)
        if (fixedVert[i] < 0 || fixedVert[i] >= nV) return fail(ctx, OC_ERR_INVALID, "oc_mesh_create: fixed vertex out of range");
    oc_mesh* m = new (std::nothrow) oc_mesh;
    if (!m) return OC_ERR_NOMEM;
    m->ctx = ctx;
    m->F.assign(F, F + 3 * (size_t)nF);
    m->fixed.assign(fixedVert, fixedVert + nFixed);
    m->Vrest.assign(V_rest, V_rest + 3 * (size_t)nV);
    m->rest.resize(8 * (size_t)nF);
    // TriMesh::computeFeatures rest constants (TriMesh.cpp:343-404)
    double surfaceArea = 0.0;
    if (!rest_constants(V_rest, F, nF, areaThres, m->rest, surfaceArea)) {
        delete m;
        return fail(ctx, OC_ERR_DEGENERATE, "oc_mesh_create: zero-area rest triangle");
    }
    double avg = 0.0;
    for (int t = 0; t < nF; ++t)
        for (int j = 0; j < 3; ++j) {
            const double* p = V_rest + 3 * (size_t)F[3 * t + j];
            const double* q = V_rest + 3 * (size_t)F[3 * t + (j + 1) % 3];
            avg += std::sqrt((p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]));
        }
    m->scalars[0] = surfaceArea;
    m->scalars[1] = avg / (3.0 * nF);
    m->scalars[2] = std::sqrt(surfaceArea / M_PI);
    std::vector<unsigned char> mask(nV, 0);
    for (int i = 0; i < nFixed; ++i) mask[fixedVert[i]] = 1;
    oc::DeviceMesh& d = m->d;
    int rc = device_mesh_upload(ctx, d, nV, F, nF, m->rest, surfaceArea, mask);
    cudaStream_t st = ctx->stream;
    auto chk = [&](cudaError_t e, const char* what) {
        if (rc == OC_OK && e != cudaSuccess) rc = fail(ctx, OC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    chk(dalloc(&d.uv, nV), "alloc");
    chk(dalloc(&m->cornerBuf, 3 * (size_t)nF), "alloc");
    chk(dalloc(&m->tmpV, nV), "alloc");
    chk(dalloc(&m->hb, 21 * (size_t)nF), "alloc");
    m->scratch.maxBlocks = oc::kMaxReduceBlocks;
    chk(dalloc(&m->scratch.partials, (size_t)m->scratch.maxBlocks * oc::kMaxTrials), "alloc");
    chk(dalloc(&m->scratch.result, 16), "alloc");
    chk(dalloc(&m->scratch.minBits, 2), "alloc");
    chk(cudaMallocHost(&m->scratch.hostResult, sizeof(double) * 16), "alloc host");
    if (rc == OC_OK) {
        chk(cudaMemcpyAsync(d.uv, UV, sizeof(double2) * nV, cudaMemcpyHostToDevice, st), "upload");
        chk(cudaStreamSynchronize(st), "sync");
    }
    if (rc != OC_OK) {
        oc_mesh_destroy(m);
        return rc;
    }
    *out = m;
    return OC_OK;
}

int oc_mesh_destroy(oc_mesh* m)
{
    if (!m) return OC_ERR_INVALID;
    device_mesh_free(m->d);
    cudaFree(m->d.uv);
    cudaFree(m->cornerBuf); cudaFree(m->tmpV); cudaFree(m->hb); cudaFree(m->tmpF); cudaFree(m->divGrad);
    cudaFree(m->scratch.partials); cudaFree(m->scratch.result); cudaFree(m->scratch.minBits);
    if (m->scratch.hostResult) cudaFreeHost(m->scratch.hostResult);
    delete m;
    return OC_OK;
}

int oc_mesh_set_uv(oc_mesh* m, const double* UV)
{
    if (!m || !UV) return OC_ERR_INVALID;
    OC_CUDA(m->ctx, cudaMemcpyAsync(m->d.uv, UV, sizeof(double2) * m->d.nV, cudaMemcpyHostToDevice, m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    return OC_OK;
}

int oc_mesh_get_uv(oc_mesh* m, double* UV)
{
    if (!m || !UV) return OC_ERR_INVALID;
    OC_CUDA(m->ctx, cudaMemcpyAsync(UV, m->d.uv, sizeof(double2) * m->d.nV, cudaMemcpyDeviceToHost, m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    return OC_OK;
}

int oc_mesh_rest_constants(oc_mesh* m, double* rest, double* scalars)
{
    if (!m) return OC_ERR_INVALID;
    if (rest) std::memcpy(rest, m->rest.data(), sizeof(double) * m->rest.size());
    if (scalars) std::memcpy(scalars, m->scalars, sizeof(m->scalars));
    return OC_OK;
}

int oc_mesh_check_inversion(oc_mesh* m, int* ok)
{
    if (!m || !ok) return OC_ERR_INVALID;
    oc::launch_check_inversion(m->d, m->scratch, m->ctx->stream);
    double bitsAsDouble;
    int rc = read_min(m, &bitsAsDouble);
    if (rc) return rc;
    unsigned long long count;
    std::memcpy(&count, &bitsAsDouble, sizeof(count));
    *ok = count == 0 ? 1 : 0;
    return OC_OK;
}

// ------------------------------------------------------------------ energy
int oc_sd_energy(oc_mesh* m, int uniformWeight, double* energyVal)
{
    if (!m || !energyVal) return OC_ERR_INVALID;
    oc::launch_energy(m->d, m->d.uv, nullptr, nullptr, 1, uniformWeight, 1.0, m->scratch, m->ctx->stream);
    return read_result(m, 1, energyVal);
}

int oc_sd_energy_per_elem(oc_mesh* m, int uniformWeight, double* out)
{
    if (!m || !out) return OC_ERR_INVALID;
    if (!m->tmpF) OC_CUDA(m->ctx, dalloc(&m->tmpF, 36 * (size_t)m->d.nF));
    oc::launch_energy_elem(m->d, uniformWeight, m->tmpF, m->ctx->stream);
    OC_CUDA(m->ctx, cudaGetLastError());
    OC_CUDA(m->ctx, cudaMemcpyAsync(out, m->tmpF, sizeof(double) * m->d.nF, cudaMemcpyDeviceToHost, m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    return OC_OK;
}

int oc_sd_gradient(oc_mesh* m, int uniformWeight, double* gradient)
{
    if (!m || !gradient) return OC_ERR_INVALID;
    oc::launch_gradient(m->d, uniformWeight, 1.0, m->cornerBuf, m->tmpV, m->scratch, m->ctx->stream);
    OC_CUDA(m->ctx, cudaGetLastError());
    OC_CUDA(m->ctx, cudaMemcpyAsync(gradient, m->tmpV, sizeof(double2) * m->d.nV, cudaMemcpyDeviceToHost, m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    return OC_OK;
}

int oc_sd_hessian_blocks(oc_mesh* m, int uniformWeight, double* blocks)
{
    return oc_sd_hessian_blocks_projected(m, uniformWeight, OC_HESSIAN_JACOBI6, blocks);
}

int oc_sd_hessian_blocks_projected(oc_mesh* m, int uniformWeight, int projection, double* blocks)
{
    if (!m || !blocks || projection < OC_HESSIAN_REDUCED || projection > OC_HESSIAN_HYBRID) return OC_ERR_INVALID;
    if (!m->tmpF) OC_CUDA(m->ctx, dalloc(&m->tmpF, 36 * (size_t)m->d.nF));
    oc::launch_hessian(m->d, uniformWeight, m->hb, m->ctx->stream, projection);
    oc::launch_hessian_expand(m->hb, m->d.nF, m->tmpF, m->ctx->stream);
    OC_CUDA(m->ctx, cudaGetLastError());
    OC_CUDA(m->ctx, cudaMemcpyAsync(blocks, m->tmpF, sizeof(double) * 36 * (size_t)m->d.nF, cudaMemcpyDeviceToHost,
                                    m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    return OC_OK;
}

int oc_sd_init_step_size(oc_mesh* m, const double* searchDir, double* stepSize)
{
    if (!m || !searchDir || !stepSize || !(*stepSize > 0.0)) return OC_ERR_INVALID;
    OC_CUDA(m->ctx, cudaMemcpyAsync(m->tmpV, searchDir, sizeof(double2) * m->d.nV, cudaMemcpyHostToDevice, m->ctx->stream));
    oc::launch_init_step(m->d, m->tmpV, *stepSize, m->scratch, m->ctx->stream);
    double s;
    int rc = read_min(m, &s);
    if (rc) return rc;
    *stepSize = s;
    return OC_OK;
}

// ------------------------------------------------------------------ topology
// Re-derives the device mesh from its host topology after an operation
// (TriMesh::computeFeatures, TriMesh.cpp:343-518): rest constants, scalars,
// corner lists; UV from uvHost.
static int mesh_rebuild(oc_mesh* m, const std::vector<double>& uvHost)
{
    oc_ctx* ctx = m->ctx;
    ++m->topoVersion;
    m->adj.reset();
    const int nV = static_cast<int>(m->Vrest.size() / 3), nF = static_cast<int>(m->F.size() / 3);
    double surfaceArea = 0.0;
    std::vector<double> rest;
    if (!rest_constants(m->Vrest.data(), m->F.data(), nF, 0.0, rest, surfaceArea))
        return fail(ctx, OC_ERR_DEGENERATE, "topology op: zero-area rest triangle");
    m->rest.swap(rest);
    double avg = 0.0;
    const double* Vr = m->Vrest.data();
    const int* F = m->F.data();
    {   // edge lengths on the host pool, summed in triangle order
        std::vector<double> el(3 * (size_t)nF);
        oc::host_parallel_for(nF, 4096, [&](size_t t0, size_t t1) {
            for (size_t t = t0; t < t1; ++t)
                for (int j = 0; j < 3; ++j) {
                    const double* p = Vr + 3 * (size_t)F[3 * t + j];
                    const double* q = Vr + 3 * (size_t)F[3 * t + (j + 1) % 3];
                    el[3 * t + j] = std::sqrt((p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) +
                                              (p[2] - q[2]) * (p[2] - q[2]));
                }
        });
        for (double x : el) avg += x;
    }
    m->scalars[0] = surfaceArea;
    m->scalars[1] = avg / (3.0 * nF);
    m->scalars[2] = std::sqrt(surfaceArea / M_PI);
    std::vector<unsigned char> mask(nV, 0);
    for (int v : m->fixed)
        if (v < nV) mask[v] = 1;
    const int oldNV = m->d.nV;
    int rc = device_mesh_upload(ctx, m->d, nV, F, nF, m->rest, surfaceArea, mask);
    if (rc) return rc;
    if (nV != oldNV) {
        cudaFree(m->d.uv); cudaFree(m->tmpV); cudaFree(m->divGrad);
        m->d.uv = nullptr; m->tmpV = nullptr; m->divGrad = nullptr;
        OC_CUDA(ctx, dalloc(&m->d.uv, nV));
        OC_CUDA(ctx, dalloc(&m->tmpV, nV));
    }
    OC_CUDA(ctx, cudaMemcpyAsync(m->d.uv, uvHost.data(), sizeof(double2) * nV, cudaMemcpyHostToDevice, ctx->stream));
    OC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return OC_OK;
}

// host edit, then the device mesh; ms2 (optional) gets the two durations
static int apply_topology(oc_mesh* m, int opType, const int* path, int pathLen, const double* newVertPos, int posRows,
                          double* ms2)
{
    if (!m || !path || !newVertPos) return OC_ERR_INVALID;
    auto t = std::chrono::steady_clock::now();
    std::vector<double> uv(2 * (size_t)m->d.nV);
    OC_CUDA(m->ctx, cudaMemcpyAsync(uv.data(), m->d.uv, sizeof(double2) * m->d.nV, cudaMemcpyDeviceToHost,
                                    m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    std::vector<int> F(m->F), cohE(m->cohE);
    std::vector<double> Vrest(m->Vrest);
    std::string err;
    int tails[3] = {m->tails[0], m->tails[1], m->tails[2]};
    int edit[3] = {-1, -1, -1};
    const int nV0 = m->d.nV;
    int rc = oc::topo_apply(opType, path, pathLen, newVertPos, posRows, F, Vrest, uv, cohE, &err, tails, edit);
    if (rc) return fail(m->ctx, rc, err);
    std::copy(tails, tails + 3, m->tails);
    m->F.swap(F);
    m->Vrest.swap(Vrest);
    m->cohE.swap(cohE);
    if (ms2) ms2[0] = ms_since(t);
    rc = mesh_rebuild(m, uv);
    if (ms2) ms2[1] = ms_since(t);
    if (rc == OC_OK && edit[0] >= 0) {
        if (m->editLog.size() >= 1024) m->editLog.erase(m->editLog.begin(), m->editLog.begin() + 512);
        m->editLog.push_back({static_cast<long long>(m->topoVersion), edit[0], edit[1], edit[2], nV0});
    }
    return rc;
}

int oc_mesh_apply_topology(oc_mesh* m, int opType, const int* path, int pathLen, const double* newVertPos, int posRows)
{
    return apply_topology(m, opType, path, pathLen, newVertPos, posRows, nullptr);
}

int oc_mesh_get_topology(oc_mesh* m, int* nV, int* nF, int* nCohE, int* F, double* Vrest, int* cohE)
{
    if (!m) return OC_ERR_INVALID;
    if (nV) *nV = m->d.nV;
    if (nF) *nF = m->d.nF;
    if (nCohE) *nCohE = static_cast<int>(m->cohE.size() / 4);
    if (F) std::copy(m->F.begin(), m->F.end(), F);
    if (Vrest) std::copy(m->Vrest.begin(), m->Vrest.end(), Vrest);
    if (cohE) std::copy(m->cohE.begin(), m->cohE.end(), cohE);
    return OC_OK;
}

int oc_mesh_set_cohesive_edges(oc_mesh* m, const int* cohE, int nCohE)
{
    if (!m || nCohE < 0 || (nCohE && !cohE)) return OC_ERR_INVALID;
    for (long long i = 0; i < 4LL * nCohE; ++i)
        if (cohE[i] < -1 || cohE[i] >= m->d.nV) return fail(m->ctx, OC_ERR_INVALID, "cohesive edge: vertex out of range");
    m->cohE.assign(cohE, cohE + 4 * (size_t)nCohE);
    return OC_OK;
}

int oc_mesh_drop_adjacency(oc_mesh* m)
{
    if (!m) return OC_ERR_INVALID;
    m->adj.reset();
    return OC_OK;
}

int oc_mesh_split_filter(oc_mesh* m, double* divGrad)
{
    if (!m || !divGrad) return OC_ERR_INVALID;
    if (!m->divGrad) OC_CUDA(m->ctx, dalloc(&m->divGrad, m->d.nV));
    oc::launch_divgrad(m->d, m->cornerBuf, m->divGrad, m->ctx->stream);
    OC_CUDA(m->ctx, cudaGetLastError());
    OC_CUDA(m->ctx, cudaMemcpyAsync(divGrad, m->divGrad, sizeof(double) * m->d.nV, cudaMemcpyDeviceToHost,
                                    m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    return OC_OK;
}

struct oc_topo_result {
    std::vector<oc::TopoCandidate> cands;
    int best = -1, pool = 0;
    oc::TopoStats stats;
    oc::TopoExtras extras;
};

static int topology_query(oc_mesh* m, int opType, double lambda_t, double filterExp, const oc::TopoOptions& opts,
                          oc_topo_result** out);

int oc_topology_query(oc_mesh* m, int opType, double lambda_t, double filterExp, int options, oc_topo_result** out)
{
    oc::TopoOptions opts;
    opts.flags = options & (oc::kTopoFp32Hessian | oc::kTopoRecordFeatures | oc::kTopoAutotune | oc::kTopoBijective);
    return topology_query(m, opType, lambda_t, filterExp, opts, out);
}

int oc_topology_query_learned(oc_mesh* m, int opType, double lambda_t, double filterExp, int options, oc_mlp* mlp,
                              double topFrac, oc_topo_result** out)
{
    if (!mlp || mlp->m.in != oc::kTopoNumFeatures || !(topFrac > 0.0) || topFrac > 1.0) return OC_ERR_INVALID;
    oc::TopoOptions opts;
    opts.flags = (options & (oc::kTopoFp32Hessian | oc::kTopoAutotune | oc::kTopoBijective)) | oc::kTopoLearned;
    opts.mlp = &mlp->m;
    opts.topFrac = topFrac;
    return topology_query(m, opType, lambda_t, filterExp, opts, out);
}

// the operations ops[0..nOps) on the mesh's current state, solved together
static int topology_queries(oc_mesh* m, const int* ops, int nOps, double lambda_t, double filterExp,
                            const oc::TopoOptions& opts, oc_topo_result** out, const int* candVerts = nullptr,
                            int nCandVerts = 0, int mergeFork = -2, int shardRank = 0, int shardCount = 1)
{
    if (!m || !out || nOps <= 0) return OC_ERR_INVALID;
    auto tPrep = std::chrono::steady_clock::now();
    bool split = false;
    for (int i = 0; i < nOps; ++i) {
        out[i] = nullptr;
        if (ops[i] < 0 || ops[i] > 2) return OC_ERR_INVALID;
        split = split || ops[i] != oc::kOpMerge;
    }
    const int nV = m->d.nV;
    std::vector<double> uv(2 * (size_t)nV), dg;
    OC_CUDA(m->ctx, cudaMemcpyAsync(uv.data(), m->d.uv, sizeof(double2) * nV, cudaMemcpyDeviceToHost, m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    if (split && !candVerts) {
        dg.resize(nV);
        int rc = oc_mesh_split_filter(m, dg.data());
        if (rc) return rc;
    }
    oc::TopoQueryIn in;
    in.nV = nV;
    in.nF = m->d.nF;
    in.F = m->F.data();
    in.Vrest = m->Vrest.data();
    in.rest = m->rest.data();
    in.UV = uv.data();
    in.cohE = m->cohE.empty() ? nullptr : m->cohE.data();
    in.nCohE = static_cast<int>(m->cohE.size() / 4);
    in.surfaceArea = m->scalars[0];
    in.avgEdgeLen = m->scalars[1];
    in.virtualRadius = m->scalars[2];
    in.divGrad = dg.empty() ? nullptr : dg.data();
    in.dm = &m->d;
    in.st = m->ctx->stream;
    if (!m->adj) m->adj = oc::topo_adjacency(nV, m->F.data(), m->d.nF);
    in.adj = m->adj.get();
    // largest cluster of blocks per local problem: the device's (16 or 8)
    // unless the OC_LOCAL_CLUSTER environment variable caps it at 1, 2, 4 or 8
    static const int bigCluster = [] {
        const char* e = std::getenv("OC_LOCAL_CLUSTER");
        const int v = e ? std::atoi(e) : 0;
        return (v == 1 || v == 2 || v == 4 || v == 8) ? v : 0;
    }();
    in.bigCluster = bigCluster;
    if (!m->topoWs) m->topoWs = std::make_shared<oc::TopoWorkspace>();
    in.ws = m->topoWs.get();
    in.candVerts = candVerts;
    in.nCandVerts = nCandVerts;
    in.mergeFork = mergeFork;
    in.shardRank = shardRank;
    in.shardCount = shardCount;
    // bijective form: the scaffold's air mesh as it stands (air-only
    // vertices where the last step moved them)
    std::vector<double> airV;
    std::vector<int> airF, airBnd;
    if (opts.flags & oc::kTopoBijective) {
        oc_optimizer* o = m->scafOwner;
        if (!o) return fail(m->ctx, OC_ERR_INVALID, "bijective topology query: the mesh has no scaffold");
        int nAirV = 0, nAirF = 0, nBnd = 0;
        int rc = oc_optimizer_get_scaffold(o, &nAirV, &nAirF, &nBnd, nullptr, nullptr, nullptr);
        if (rc) return rc;
        airV.resize(2 * (size_t)nAirV);
        airF.resize(3 * (size_t)nAirF);
        airBnd.resize(nBnd);
        rc = oc_optimizer_get_scaffold(o, nullptr, nullptr, nullptr, airV.data(), airF.data(), airBnd.data());
        if (rc) return rc;
        in.bijective = true;
        in.airV = airV.data();
        in.airF = airF.data();
        in.airBnd = airBnd.data();
        in.nAirV = nAirV;
        in.nAirF = nAirF;
        in.nAirBnd = nBnd;
    }
    std::vector<oc::TopoOpResult> res(nOps);
    std::string err;
    const double prepMs = ms_since(tPrep);
    const int rc = oc::topo_query_ops(in, ops, nOps, lambda_t, filterExp > 0.0 ? filterExp : 0.6, opts, res.data(),
                                      &err);
    if (rc) return fail(m->ctx, rc, err);
    for (int i = 0; i < nOps; ++i) res[i].stats.prepMs = prepMs;
    for (int i = 0; i < nOps; ++i) {
        oc_topo_result* r = new (std::nothrow) oc_topo_result;
        if (!r) {
            for (int j = 0; j < i; ++j) {
                delete out[j];
                out[j] = nullptr;
            }
            return OC_ERR_NOMEM;
        }
        r->cands.swap(res[i].cands);
        r->best = res[i].best;
        r->pool = res[i].pool;
        r->stats = res[i].stats;
        r->extras = std::move(res[i].extras);
        out[i] = r;
    }
    return OC_OK;
}

static int topology_query(oc_mesh* m, int opType, double lambda_t, double filterExp, const oc::TopoOptions& opts,
                          oc_topo_result** out)
{
    if (!m || !out || opType < 0 || opType > 2) return OC_ERR_INVALID;
    return topology_queries(m, &opType, 1, lambda_t, filterExp, opts, out);
}

int oc_topology_step(oc_mesh* m, double lambda_t, double filterExp, int options, oc_mlp* mlp, double topFrac,
                     oc_topo_result** split, oc_topo_result** merge, oc_topo_result** interior)
{
    if (!split || !merge || !interior) return OC_ERR_INVALID;
    if (mlp && (mlp->m.in != oc::kTopoNumFeatures || !(topFrac > 0.0) || topFrac > 1.0)) return OC_ERR_INVALID;
    oc::TopoOptions opts;
    opts.flags = options & (oc::kTopoFp32Hessian | oc::kTopoRecordFeatures | oc::kTopoAutotune | oc::kTopoBijective);
    if (mlp) {
        opts.flags = (options & (oc::kTopoFp32Hessian | oc::kTopoAutotune | oc::kTopoBijective)) | oc::kTopoLearned;
        opts.mlp = &mlp->m;
        opts.topFrac = topFrac;
    }
    const int ops[3] = {oc::kOpBoundarySplit, oc::kOpMerge, oc::kOpInteriorSplit};
    oc_topo_result* r[3] = {};
    const int rc = topology_queries(m, ops, 3, lambda_t, filterExp, opts, r);
    if (rc) return rc;
    *split = r[0];
    *merge = r[1];
    *interior = r[2];
    return OC_OK;
}

int oc_topology_queries(oc_mesh* m, const int* ops, int nOps, double lambda_t, double filterExp, int options,
                        oc_mlp* mlp, double topFrac, oc_topo_result** out)
{
    if (!ops || !out || nOps <= 0 || nOps > 3) return OC_ERR_INVALID;
    if (mlp && (mlp->m.in != oc::kTopoNumFeatures || !(topFrac > 0.0) || topFrac > 1.0)) return OC_ERR_INVALID;
    oc::TopoOptions opts;
    opts.flags = options & (oc::kTopoFp32Hessian | oc::kTopoRecordFeatures | oc::kTopoAutotune | oc::kTopoBijective);
    if (mlp) {
        opts.flags = (options & (oc::kTopoFp32Hessian | oc::kTopoAutotune | oc::kTopoBijective)) | oc::kTopoLearned;
        opts.mlp = &mlp->m;
        opts.topFrac = topFrac;
    }
    return topology_queries(m, ops, nOps, lambda_t, filterExp, opts, out);
}

int oc_topology_queries_sharded(oc_mesh* m, const int* ops, int nOps, double lambda_t, double filterExp, int options,
                                oc_mlp* mlp, double topFrac, int shardRank, int shardCount, oc_topo_result** out)
{
    if (!ops || !out || nOps <= 0 || nOps > 3 || shardCount < 1 || shardRank < 0 || shardRank >= shardCount)
        return OC_ERR_INVALID;
    if (mlp && (mlp->m.in != oc::kTopoNumFeatures || !(topFrac > 0.0) || topFrac > 1.0)) return OC_ERR_INVALID;
    oc::TopoOptions opts;
    opts.flags = options & (oc::kTopoFp32Hessian | oc::kTopoRecordFeatures | oc::kTopoAutotune | oc::kTopoBijective);
    if (mlp) {
        opts.flags = (options & (oc::kTopoFp32Hessian | oc::kTopoAutotune | oc::kTopoBijective)) | oc::kTopoLearned;
        opts.mlp = &mlp->m;
        opts.topFrac = topFrac;
    }
    return topology_queries(m, ops, nOps, lambda_t, filterExp, opts, out, nullptr, 0, -2, shardRank, shardCount);
}

int oc_topology_query_tail(oc_mesh* m, int opType, double lambda_t, int options, oc_topo_result** out)
{
    // querySplit / queryMerge with propagate = true (TriMesh.cpp:637-665,
    // 828-833): boundary splits at the current fracture tail (or at the two
    // ends of the last interior split), merges of the pair forking there
    if (!m || !out || (opType != oc::kOpBoundarySplit && opType != oc::kOpMerge)) return OC_ERR_INVALID;
    oc::TopoOptions opts;
    opts.flags = options & (oc::kTopoFp32Hessian | oc::kTopoBijective);
    if (opType == oc::kOpMerge) return topology_queries(m, &opType, 1, lambda_t, 0.6, opts, out, nullptr, 0, m->tails[0]);
    int verts[2] = {-1, -1};
    int n = 0;
    if (m->tails[0] >= 0) verts[n++] = m->tails[0];
    else if (m->tails[1] >= 0) {
        verts[n++] = m->tails[1];
        verts[n++] = m->tails[2];
    }
    return topology_queries(m, &opType, 1, lambda_t, 0.6, opts, out, verts, n);
}

int oc_topology_schedules(int* nRows, int* rows, float* ms)
{
    if (!nRows) return OC_ERR_INVALID;
    const auto t = oc::topo_schedule_table();
    *nRows = static_cast<int>(t.size());
    for (size_t i = 0; i < t.size(); ++i) {
        const oc::ScheduleRecord& r = t[i];
        if (rows) {
            const int v[11] = {r.device, r.cls, r.countBucket, r.triBucket, r.best.tpp, r.best.cluster, r.best.block,
                               r.rule.tpp, r.rule.cluster, r.rule.block, r.candidates};
            std::copy(v, v + 11, rows + 11 * i);
        }
        if (ms) {
            ms[2 * i] = r.bestMs;
            ms[2 * i + 1] = r.ruleMs;
        }
    }
    return OC_OK;
}

int oc_mesh_fracture_tails(oc_mesh* m, int* tails3)
{
    if (!m || !tails3) return OC_ERR_INVALID;
    std::copy(m->tails, m->tails + 3, tails3);
    return OC_OK;
}

int oc_mesh_set_fracture_tails(oc_mesh* m, const int* tails3)
{
    if (!m || !tails3) return OC_ERR_INVALID;
    for (int k = 0; k < 3; ++k)
        if (tails3[k] < -1 || tails3[k] >= m->d.nV) return fail(m->ctx, OC_ERR_INVALID, "fracture tail out of range");
    std::copy(tails3, tails3 + 3, m->tails);
    return OC_OK;
}

int oc_mesh_seam_length(oc_mesh* m, double* seamLen)
{
    // TriMesh::computeSeamSparsity (TriMesh.cpp:1542-1558), triSoup off and
    // no initial seam length: rest length of every interior cohesive pair
    if (!m || !seamLen) return OC_ERR_INVALID;
    double s = 0.0;
    const double* Vr = m->Vrest.data();
    for (size_t r = 0; r < m->cohE.size() / 4; ++r) {
        const int* c = &m->cohE[4 * r];
        if (std::min(std::min(c[0], c[1]), std::min(c[2], c[3])) < 0) continue;
        const double dx = Vr[3 * (size_t)c[0]] - Vr[3 * (size_t)c[1]];
        const double dy = Vr[3 * (size_t)c[0] + 1] - Vr[3 * (size_t)c[1] + 1];
        const double dz = Vr[3 * (size_t)c[0] + 2] - Vr[3 * (size_t)c[1] + 2];
        s += std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    *seamLen = s;
    return OC_OK;
}

int oc_topo_result_info(const oc_topo_result* r, int* nCand, int* best, int* pool, int* nProblems, int* maxIters,
                        double* buildMs, double* solveMs)
{
    if (!r) return OC_ERR_INVALID;
    if (nCand) *nCand = static_cast<int>(r->cands.size());
    if (best) *best = r->best;
    if (pool) *pool = r->pool;
    if (nProblems) *nProblems = r->stats.nProblems;
    if (maxIters) *maxIters = r->stats.maxIters;
    if (buildMs) *buildMs = r->stats.buildMs;
    if (solveMs) *solveMs = r->stats.solveMs;
    return OC_OK;
}

int oc_topo_result_timing(const oc_topo_result* r, int* nSelected, double* probeMs, double* exactMs)
{
    if (!r) return OC_ERR_INVALID;
    if (nSelected) *nSelected = r->stats.nSelected;
    if (probeMs) *probeMs = r->stats.probeMs;
    if (exactMs) *exactMs = r->stats.exactMs;
    return OC_OK;
}

int oc_topo_result_host_phases(const oc_topo_result* r, double* out4)
{
    if (!r || !out4) return OC_ERR_INVALID;
    out4[0] = r->stats.prepMs;
    out4[1] = r->stats.airMs;
    out4[2] = r->stats.rankMs;
    out4[3] = r->stats.finishMs;
    return OC_OK;
}

int oc_topo_result_features(const oc_topo_result* r, int* nRows, float* X, float* target, float* predicted)
{
    if (!r || !nRows) return OC_ERR_INVALID;
    *nRows = static_cast<int>(r->extras.X.size() / oc::kTopoNumFeatures);
    if (X) std::copy(r->extras.X.begin(), r->extras.X.end(), X);
    if (target) std::copy(r->extras.target.begin(), r->extras.target.end(), target);
    if (predicted) std::copy(r->extras.predicted.begin(), r->extras.predicted.end(), predicted);
    return OC_OK;
}

int oc_topo_result_problems(const oc_topo_result* r, int* nProblems, int* cand, double* ewExact, double* ewPred)
{
    if (!r || !nProblems) return OC_ERR_INVALID;
    const auto& x = r->extras;
    *nProblems = static_cast<int>(x.cand.size());
    if (cand) std::copy(x.cand.begin(), x.cand.end(), cand);
    if (ewExact) std::copy(x.ewExact.begin(), x.ewExact.end(), ewExact);
    if (ewPred) {
        if (x.ewPred.size() == x.cand.size()) std::copy(x.ewPred.begin(), x.ewPred.end(), ewPred);
        else std::fill(ewPred, ewPred + x.cand.size(), std::nan(""));
    }
    return OC_OK;
}

int oc_topo_result_problem_stats(const oc_topo_result* r, int* nProblems, int* nTri, int* nFree, int* iters,
                                 int* trials, long long* cycles)
{
    if (!r || !nProblems) return OC_ERR_INVALID;
    const auto& x = r->extras;
    *nProblems = static_cast<int>(x.nTri.size());
    if (nTri) std::copy(x.nTri.begin(), x.nTri.end(), nTri);
    if (nFree) std::copy(x.nFree.begin(), x.nFree.end(), nFree);
    if (iters) std::copy(x.iters.begin(), x.iters.end(), iters);
    if (trials) std::copy(x.trials.begin(), x.trials.end(), trials);
    if (cycles) std::copy(x.cycles.begin(), x.cycles.end(), cycles);
    return OC_OK;
}

int oc_topo_result_iterations(const oc_topo_result* r, int* totalIters, int* capped, long long* trials)
{
    if (!r) return OC_ERR_INVALID;
    if (totalIters) *totalIters = r->stats.totalIters;
    if (capped) *capped = r->stats.nonConverged;
    if (trials) *trials = r->stats.totalTrials;
    return OC_OK;
}

int oc_topo_result_candidate(const oc_topo_result* r, int c, double* EwDec, double* energyChanges, int* path,
                             int* pathLen, double* newVertPos, int* posRows)
{
    if (!r || c < 0 || c >= (int)r->cands.size()) return OC_ERR_INVALID;
    const oc::TopoCandidate& C = r->cands[c];
    if (EwDec) *EwDec = C.EwDec;
    if (energyChanges) { energyChanges[0] = C.ec0; energyChanges[1] = C.ec1; }
    if (pathLen) *pathLen = static_cast<int>(C.path.size());
    if (path) std::copy(C.path.begin(), C.path.end(), path);
    if (posRows) *posRows = static_cast<int>(C.pos.size() / 2);
    if (newVertPos) std::copy(C.pos.begin(), C.pos.end(), newVertPos);
    return OC_OK;
}

int oc_topo_result_candidates(const oc_topo_result* r, double* EwDec, double* energyChanges, int* path,
                              double* newVertPos, int* posRows)
{
    if (!r) return OC_ERR_INVALID;
    for (size_t c = 0; c < r->cands.size(); ++c) {
        const oc::TopoCandidate& C = r->cands[c];
        if (EwDec) EwDec[c] = C.EwDec;
        if (energyChanges) { energyChanges[2 * c] = C.ec0; energyChanges[2 * c + 1] = C.ec1; }
        if (path)
            for (int k = 0; k < 3; ++k) path[3 * c + k] = k < (int)C.path.size() ? C.path[k] : -1;
        if (newVertPos)
            for (int k = 0; k < 8; ++k) newVertPos[8 * c + k] = k < (int)C.pos.size() ? C.pos[k] : 0.0;
        if (posRows) posRows[c] = static_cast<int>(C.pos.size() / 2);
    }
    return OC_OK;
}

int oc_topology_split_candidates(int nV, const int* F, int nF, const double* divGrad, int interior, double filterExp,
                                 int* cands, int* nCands, int* pool)
{
    if (nV <= 0 || nF <= 0 || !F || !divGrad || !nCands) return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return OC_ERR_INVALID;
    std::vector<int> c;
    int p = 0;
    oc::topo_split_candidates(nV, F, nF, divGrad, interior != 0, filterExp > 0.0 ? filterExp : 0.6, c, p);
    if (cands) std::copy(c.begin(), c.end(), cands);
    *nCands = static_cast<int>(c.size());
    if (pool) *pool = p;
    return OC_OK;
}

int oc_topology_apply(int opType, const int* path, int pathLen, const double* newVertPos, int posRows, int nV, int nF,
                      const int* F, const double* Vrest, const double* UV, int nCohE, const int* cohE, int* F_out,
                      double* Vrest_out, double* UV_out, int* cohE_out, int* nV_out, int* nCohE_out)
{
    if (nV <= 0 || nF <= 0 || !F || !Vrest || !UV || nCohE < 0 || (nCohE && !cohE) || !F_out || !Vrest_out ||
        !UV_out || !nV_out || !nCohE_out)
        return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return OC_ERR_INVALID;
    std::vector<int> f(F, F + 3 * (size_t)nF), c(cohE, cohE + 4 * (size_t)nCohE);
    std::vector<double> vr(Vrest, Vrest + 3 * (size_t)nV), uv(UV, UV + 2 * (size_t)nV);
    const int rc = oc::topo_apply(opType, path, pathLen, newVertPos, posRows, f, vr, uv, c, nullptr);
    if (rc) return rc;
    std::copy(f.begin(), f.end(), F_out);
    std::copy(vr.begin(), vr.end(), Vrest_out);
    std::copy(uv.begin(), uv.end(), UV_out);
    if (cohE_out) std::copy(c.begin(), c.end(), cohE_out);
    *nV_out = static_cast<int>(uv.size() / 2);
    *nCohE_out = static_cast<int>(c.size() / 4);
    return OC_OK;
}

int oc_topology_cut_path(const int* path, int pathLen, int nV, int nF, const int* F, const double* Vrest,
                         const double* UV, int nCohE, const int* cohE, int* F_out, double* Vrest_out, double* UV_out,
                         int* cohE_out, int* nV_out, int* nCohE_out, int* nSplit)
{
    if (!path || pathLen < 2 || nV <= 0 || nF <= 0 || !F || !Vrest || !UV || nCohE < 0 || (nCohE && !cohE) ||
        !F_out || !Vrest_out || !UV_out || !nV_out || !nCohE_out)
        return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return OC_ERR_INVALID;
    std::vector<int> f(F, F + 3 * (size_t)nF), c(cohE, cohE + 4 * (size_t)nCohE);
    std::vector<double> vr(Vrest, Vrest + 3 * (size_t)nV), uv(UV, UV + 2 * (size_t)nV);
    int made = 0;
    const int rc = oc::topo_cut_path(path, pathLen, f, vr, uv, c, made, nullptr);
    if (rc) return rc;
    std::copy(f.begin(), f.end(), F_out);
    std::copy(vr.begin(), vr.end(), Vrest_out);
    std::copy(uv.begin(), uv.end(), UV_out);
    if (cohE_out) std::copy(c.begin(), c.end(), cohE_out);
    *nV_out = static_cast<int>(uv.size() / 2);
    *nCohE_out = static_cast<int>(c.size() / 4);
    if (nSplit) *nSplit = made;
    return OC_OK;
}

int oc_cut_to_disk(const int* F, int nF, int* cutVerts, int capVerts, int* cutOff, int capCuts, int* nCuts,
                   int* nVerts)
{
    if (nF < 0 || (nF && !F) || !nCuts || !nVerts) return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0) return OC_ERR_INVALID;
    std::vector<std::vector<int>> cuts;
    oc::topo_cut_to_disk(F, nF, cuts);
    long long total = 0;
    for (const auto& c : cuts) total += static_cast<long long>(c.size());
    *nCuts = static_cast<int>(cuts.size());
    *nVerts = static_cast<int>(total);
    if (!cutVerts || !cutOff) return OC_OK;   // sizes only
    if (capCuts < *nCuts + 1 || capVerts < total) return OC_ERR_INVALID;
    int o = 0;
    cutOff[0] = 0;
    for (size_t i = 0; i < cuts.size(); ++i) {
        std::copy(cuts[i].begin(), cuts[i].end(), cutVerts + o);
        o += static_cast<int>(cuts[i].size());
        cutOff[i + 1] = o;
    }
    return OC_OK;
}

int oc_topo_result_air(const oc_topo_result* r, int* problems, int* rejected, int* steinerMax, int* capped)
{
    if (!r) return OC_ERR_INVALID;
    if (problems) *problems = r->stats.airProblems;
    if (rejected) *rejected = r->stats.airRejected;
    if (steinerMax) *steinerMax = r->stats.airSteinerMax;
    if (capped) *capped = r->stats.airCapped;
    return OC_OK;
}

int oc_topo_result_destroy(oc_topo_result* r)
{
    if (!r) return OC_ERR_INVALID;
    delete r;
    return OC_OK;
}

// ------------------------------------------------------------------ linsys
int oc_linsys_create(oc_ctx* ctx, oc_linsys** out)
{
    if (!ctx || !out) return OC_ERR_INVALID;
    oc_linsys* ls = new (std::nothrow) oc_linsys;
    if (!ls) return OC_ERR_NOMEM;
    ls->ctx = ctx;
    *out = ls;
    return OC_OK;
}

int oc_linsys_destroy(oc_linsys* ls)
{
    if (!ls) return OC_ERR_INVALID;
    free_bsr(ls->b);
    oc::pcg_free(ls->wk);
    oc::chol_destroy(ls->chol);
    cudaFree(ls->dFlag); cudaFree(ls->tmpIn); cudaFree(ls->tmpOut);
    delete ls;
    return OC_OK;
}

int oc_linsys_set_type(oc_linsys* ls, int kind)
{
    if (!ls || (kind != OC_SOLVER_DIRECT && kind != OC_SOLVER_PCG)) return OC_ERR_INVALID;
    ls->kind = kind;
    return OC_OK;
}

int oc_linsys_analyze_pattern(oc_linsys* ls)
{
    if (!ls || !ls->patternSet) return OC_ERR_INVALID;
    if (ls->kind != OC_SOLVER_DIRECT || ls->chol.onDevice) return OC_OK;
    oc::chol_analyze(ls->chol, ls->nV, ls->rowPtr.data(), ls->col.data());
    std::string err;
    int rc = oc::chol_upload(ls->chol, &err);
    return rc ? fail(ls->ctx, rc, err) : OC_OK;
}

int oc_linsys_set_solve_cluster(oc_linsys* ls, int maxCluster)
{
    if (!ls || maxCluster < 1 || maxCluster > 8) return OC_ERR_INVALID;
    oc::chol_set_solve_cluster(ls->chol, maxCluster);
    return OC_OK;
}

int oc_linsys_set_factor_streams(oc_linsys* ls, int streams)
{
    if (!ls || streams < 1 || streams > oc::CholPlan::kMaxFactStreams) return OC_ERR_INVALID;
    oc::chol_set_factor_streams(ls->chol, streams);
    return OC_OK;
}

int oc_linsys_factor_streams(oc_linsys* ls, int* streams, int* groups)
{
    if (!ls || !streams || !groups) return OC_ERR_INVALID;
    const bool direct = ls->kind == OC_SOLVER_DIRECT && ls->patternSet;
    *streams = direct ? ls->chol.nFactStreams : 1;
    *groups = direct ? static_cast<int>(ls->chol.grpStream.size()) : 0;
    return OC_OK;
}

int oc_linsys_solve_clusters(oc_linsys* ls, int* levels, int* largest)
{
    if (!ls || !levels || !largest) return OC_ERR_INVALID;
    *levels = ls->kind == OC_SOLVER_DIRECT ? oc::chol_solve_cluster_levels(ls->chol, largest) : 0;
    if (ls->kind != OC_SOLVER_DIRECT) *largest = 1;
    return OC_OK;
}

static void chol_stats(const oc::CholPlan& P, double* out)
{
    double entries = 0.0;
    for (int f = 0; f < P.nFronts; ++f) entries += (double)P.fm[f] * P.fk[f];
    out[0] = P.nFronts;
    out[1] = P.nLevels;
    out[2] = P.maxM;
    out[3] = (double)P.poolSize;
    out[4] = P.flops;
    out[5] = (double)P.launches.size();
    out[6] = entries;
    out[7] = P.nDof;
}

int oc_linsys_stats(oc_linsys* ls, double* out8)
{
    if (!ls || !out8 || !ls->patternSet || ls->kind != OC_SOLVER_DIRECT) return OC_ERR_INVALID;
    chol_stats(ls->chol, out8);
    return OC_OK;
}

int oc_chol_analyze_groups(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize,
                           int maxStreams, int* out3)
{
    if (nV <= 0 || nF < 0 || (nF && !F) || nFixed < 0 || (nFixed && !fixedVert) || !out3 || maxStreams < 1 ||
        maxStreams > oc::CholPlan::kMaxFactStreams)
        return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return OC_ERR_INVALID;
    std::vector<unsigned char> mask(nV, 0);
    for (int i = 0; i < nFixed; ++i) {
        if (fixedVert[i] < 0 || fixedVert[i] >= nV) return OC_ERR_INVALID;
        mask[fixedVert[i]] = 1;
    }
    std::vector<int> rowPtr, col, diagSlot, cPtr, cIdx;
    build_pattern(nV, F, nF, mask, rowPtr, col, diagSlot, cPtr, cIdx);
    oc::CholPlan P;
    oc::chol_set_factor_streams(P, maxStreams);
    oc::chol_analyze(P, nV, rowPtr.data(), col.data(), leafSize > 0 ? leafSize : 16);
    out3[0] = P.nFactStreams;
    out3[1] = static_cast<int>(P.grpStream.size());
    out3[2] = oc::chol_groups_ordered(P) ? 1 : 0;
    return P.valid ? OC_OK : OC_ERR_INVALID;
}

int oc_chol_analyze_stats(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize, double* out8)
{
    return oc_chol_analyze_stats_xy(nV, F, nF, fixedVert, nFixed, leafSize, nullptr, out8);
}

int oc_chol_analyze_stats_xy(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize,
                             const double* xy, double* out8)
{
    if (nV <= 0 || nF < 0 || (nF && !F) || nFixed < 0 || (nFixed && !fixedVert) || !out8) return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return OC_ERR_INVALID;
    std::vector<unsigned char> mask(nV, 0);
    for (int i = 0; i < nFixed; ++i) {
        if (fixedVert[i] < 0 || fixedVert[i] >= nV) return OC_ERR_INVALID;
        mask[fixedVert[i]] = 1;
    }
    std::vector<int> rowPtr, col, diagSlot, cPtr, cIdx;
    build_pattern(nV, F, nF, mask, rowPtr, col, diagSlot, cPtr, cIdx);
    oc::CholPlan P;
    oc::chol_analyze(P, nV, rowPtr.data(), col.data(), leafSize > 0 ? leafSize : 16, nullptr, xy);
    chol_stats(P, out8);
    return P.valid ? OC_OK : OC_ERR_INVALID;
}

int oc_chol_analyze_order(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize, int* order)
{
    if (!order) return OC_ERR_INVALID;
    if (nV <= 0 || nF < 0 || (nF && !F) || nFixed < 0 || (nFixed && !fixedVert)) return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return OC_ERR_INVALID;
    std::vector<unsigned char> mask(nV, 0);
    for (int i = 0; i < nFixed; ++i) {
        if (fixedVert[i] < 0 || fixedVert[i] >= nV) return OC_ERR_INVALID;
        mask[fixedVert[i]] = 1;
    }
    std::vector<int> rowPtr, col, diagSlot, cPtr, cIdx;
    build_pattern(nV, F, nF, mask, rowPtr, col, diagSlot, cPtr, cIdx);
    oc::CholPlan P;
    oc::chol_analyze(P, nV, rowPtr.data(), col.data(), leafSize > 0 ? leafSize : 16);
    std::copy(P.vertOrder.begin(), P.vertOrder.end(), order);
    return P.valid ? OC_OK : OC_ERR_INVALID;
}

int oc_linsys_set_pattern(oc_linsys* ls, int nV, const int* F, int nF, const int* fixedVert, int nFixed)
{
    if (!ls || nV <= 0 || nF < 0 || (nF && !F) || nFixed < 0 || (nFixed && !fixedVert)) return OC_ERR_INVALID;
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return fail(ls->ctx, OC_ERR_INVALID, "set_pattern: vertex index out of range");
    std::vector<unsigned char> mask(nV, 0);
    for (int i = 0; i < nFixed; ++i) {
        if (fixedVert[i] < 0 || fixedVert[i] >= nV) return fail(ls->ctx, OC_ERR_INVALID, "set_pattern: fixed vertex out of range");
        mask[fixedVert[i]] = 1;
    }
    return linsys_set_pattern(ls, nV, F, nF, mask);
}

int oc_linsys_set_pattern_neighbors(oc_linsys* ls, int nV, const int* nbPtr, const int* nbIdx, const int* fixedVert,
                                   int nFixed)
{
    // LinSysSolver::set_pattern(vNeighbor, fixedVert) (LinSysSolver.hpp:37-135)
    if (!ls || nV <= 0 || !nbPtr || nFixed < 0 || (nFixed && !fixedVert)) return OC_ERR_INVALID;
    if (nbPtr[0] != 0) return fail(ls->ctx, OC_ERR_INVALID, "set_pattern: neighbour offsets must start at 0");
    for (int v = 0; v < nV; ++v)
        if (nbPtr[v + 1] < nbPtr[v]) return fail(ls->ctx, OC_ERR_INVALID, "set_pattern: decreasing neighbour offsets");
    if (nbPtr[nV] && !nbIdx) return OC_ERR_INVALID;
    for (int p = 0; p < nbPtr[nV]; ++p)
        if (nbIdx[p] < 0 || nbIdx[p] >= nV) return fail(ls->ctx, OC_ERR_INVALID, "set_pattern: neighbour out of range");
    std::vector<unsigned char> mask(nV, 0);
    for (int i = 0; i < nFixed; ++i) {
        if (fixedVert[i] < 0 || fixedVert[i] >= nV) return fail(ls->ctx, OC_ERR_INVALID, "set_pattern: fixed vertex out of range");
        mask[fixedVert[i]] = 1;
    }
    return linsys_set_pattern(ls, nV, nullptr, 0, mask, nullptr, 0, nullptr, nullptr, nullptr, nbPtr, nbIdx);
}

int oc_linsys_update_a(oc_linsys* ls, const int* I, const int* J, const double* V, int n)
{
    if (!ls || !ls->patternSet || n < 0 || (n && (!I || !J || !V))) return OC_ERR_INVALID;
    const int nV = ls->nV;
    std::vector<oc::Blk2> host(ls->b.nnzb, oc::Blk2{0.0, 0.0, 0.0, 0.0});
    std::vector<double> acc(4 * (size_t)ls->b.nnzb, 0.0);
    auto slot = [&](int r, int c) -> int {
        const int* lo = ls->col.data() + ls->rowPtr[r];
        const int* hi = ls->col.data() + ls->rowPtr[r + 1];
        const int* f = std::lower_bound(lo, hi, c);
        return (f != hi && *f == c) ? static_cast<int>(f - ls->col.data()) : -1;
    };
    for (int k = 0; k < n; ++k) {
        const int i = I[k], j = J[k];
        if (i < 0 || j < 0 || i >= 2 * nV || j >= 2 * nV) return fail(ls->ctx, OC_ERR_INVALID, "update_a: index out of range");
        if (i > j) continue;   // LinSysSolver.hpp:150 keeps i <= j
        const int s = slot(i / 2, j / 2);
        if (s < 0) return fail(ls->ctx, OC_ERR_INVALID, "update_a: entry outside the pattern");
        acc[4 * (size_t)s + 2 * (i & 1) + (j & 1)] += V[k];
        if (i != j) {
            const int s2 = slot(j / 2, i / 2);
            acc[4 * (size_t)s2 + 2 * (j & 1) + (i & 1)] += V[k];
        }
    }
    for (int s = 0; s < ls->b.nnzb; ++s)
        host[s] = oc::Blk2{acc[4 * (size_t)s], acc[4 * (size_t)s + 1], acc[4 * (size_t)s + 2], acc[4 * (size_t)s + 3]};
    OC_CUDA(ls->ctx, upload(ls->b.val, host.data(), host.size(), ls->ctx->stream));
    OC_CUDA(ls->ctx, cudaStreamSynchronize(ls->ctx->stream));
    return OC_OK;
}

int oc_linsys_factorize(oc_linsys* ls)
{
    if (!ls || !ls->patternSet) return OC_ERR_INVALID;
    int bad = 0;
    int rc = linsys_factor(ls, -1.0, &bad);
    if (rc) return rc;
    return bad ? fail(ls->ctx, OC_ERR_NOT_SPD, "factorize: non-positive pivot or diagonal block") : OC_OK;
}

int oc_linsys_solve(oc_linsys* ls, const double* rhs, double* result, double tol, int maxIter, int* iters,
                    double* relres)
{
    if (!ls || !ls->patternSet || !rhs || !result) return OC_ERR_INVALID;
    if (!(tol > 0.0)) tol = 1e-8;
    if (maxIter <= 0) maxIter = 20000;
    cudaStream_t st = ls->ctx->stream;
    OC_CUDA(ls->ctx, cudaMemcpyAsync(ls->tmpIn, rhs, sizeof(double2) * ls->nV, cudaMemcpyHostToDevice, st));
    std::string err;
    int rc;
    if (ls->kind == OC_SOLVER_DIRECT) {
        rc = oc::chol_solve(ls->chol, ls->tmpIn, ls->tmpOut, 1.0, st, &err);
        if (rc) return fail(ls->ctx, rc, err);
        if (iters) *iters = 0;
    }
    else {
        rc = oc::pcg_solve(ls->b, ls->tmpIn, ls->tmpOut, ls->wk, tol, maxIter, 1.0, st, iters, relres, &err);
        if (rc == OC_ERR_CUDA) return fail(ls->ctx, rc, err);
    }
    OC_CUDA(ls->ctx, cudaMemcpyAsync(result, ls->tmpOut, sizeof(double2) * ls->nV, cudaMemcpyDeviceToHost, st));
    OC_CUDA(ls->ctx, cudaStreamSynchronize(st));
    if (ls->kind == OC_SOLVER_DIRECT && relres) {
        // relative residual ||rhs - A x|| / ||rhs|| of the computed solution
        oc::launch_spmv(ls->b, ls->tmpOut, ls->tmpIn, st);
        std::vector<double> ax(2 * (size_t)ls->nV);
        OC_CUDA(ls->ctx, cudaMemcpyAsync(ax.data(), ls->tmpIn, sizeof(double2) * ls->nV, cudaMemcpyDeviceToHost, st));
        OC_CUDA(ls->ctx, cudaStreamSynchronize(st));
        double rr = 0.0, bb = 0.0;
        for (size_t i = 0; i < ax.size(); ++i) {
            rr += (rhs[i] - ax[i]) * (rhs[i] - ax[i]);
            bb += rhs[i] * rhs[i];
        }
        *relres = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    }
    return rc;
}

int oc_linsys_multiply(oc_linsys* ls, const double* x, double* Ax)
{
    if (!ls || !ls->patternSet || !x || !Ax) return OC_ERR_INVALID;
    OC_CUDA(ls->ctx, cudaMemcpyAsync(ls->tmpIn, x, sizeof(double2) * ls->nV, cudaMemcpyHostToDevice, ls->ctx->stream));
    oc::launch_spmv(ls->b, ls->tmpIn, ls->tmpOut, ls->ctx->stream);
    OC_CUDA(ls->ctx, cudaGetLastError());
    OC_CUDA(ls->ctx, cudaMemcpyAsync(Ax, ls->tmpOut, sizeof(double2) * ls->nV, cudaMemcpyDeviceToHost, ls->ctx->stream));
    OC_CUDA(ls->ctx, cudaStreamSynchronize(ls->ctx->stream));
    return OC_OK;
}

// ------------------------------------------------------------------ optimizer
int oc_optimizer_default_config(oc_optimizer_config* c)
{
    if (!c) return OC_ERR_INVALID;
    c->pcgTol = 1e-8;
    c->pcgMaxIter = 20000;
    c->relGL2Tol = 1e-12;
    c->lineSearchBatch = 4;
    c->timing = 0;
    c->linearSolver = OC_SOLVER_DIRECT;
    c->scaffoldPattern = 0;
    c->hessianProjection = OC_HESSIAN_JACOBI6;
    c->ordering = OC_ORDER_AUTO;
    c->carryAnalysis = 1;
    return OC_OK;
}

int oc_optimizer_create(oc_mesh* mesh, double energyParam, const oc_optimizer_config* cfg, oc_optimizer** out)
{
    if (!mesh || !out || !(energyParam > 0.0)) return OC_ERR_INVALID;
    oc_optimizer* o = new (std::nothrow) oc_optimizer;
    if (!o) return OC_ERR_NOMEM;
    o->mesh = mesh;
    o->param = energyParam;
    o->wScaf = energyParam * 0.01;   // w_scaf, fixed at construction (Optimizer.cpp:87)
    o->nWhole = o->nWholeReal = o->capWhole = mesh->d.nV;
    o->nV0 = mesh->d.nV;
    o->nFixed0 = static_cast<int>(mesh->fixed.size());
    if (cfg) o->cfg = *cfg;
    else oc_optimizer_default_config(&o->cfg);
    if (!(o->cfg.pcgTol > 0.0)) o->cfg.pcgTol = 1e-8;
    if (o->cfg.pcgMaxIter <= 0) o->cfg.pcgMaxIter = 20000;
    if (!(o->cfg.relGL2Tol > 0.0)) o->cfg.relGL2Tol = 1e-12;
    o->cfg.lineSearchBatch = std::max(1, std::min(o->cfg.lineSearchBatch, oc::kMaxTrials));
    o->relGL2Tol = o->cfg.relGL2Tol;
    oc_ctx* ctx = mesh->ctx;
    const int nV = mesh->d.nV;
    int rc = OC_OK;
    if (dalloc(&o->g, nV) != cudaSuccess || dalloc(&o->dir, nV) != cudaSuccess || dalloc(&o->uv0, nV) != cudaSuccess)
        rc = fail(ctx, OC_ERR_CUDA, "optimizer alloc");
    if (o->cfg.linearSolver != OC_SOLVER_PCG) o->cfg.linearSolver = OC_SOLVER_DIRECT;
    if (o->cfg.hessianProjection < OC_HESSIAN_REDUCED || o->cfg.hessianProjection > OC_HESSIAN_HYBRID)
        o->cfg.hessianProjection = OC_HESSIAN_JACOBI6;
    if (o->cfg.ordering != OC_ORDER_BFS) o->cfg.ordering = OC_ORDER_AUTO;
    if (rc == OC_OK) rc = oc_linsys_create(ctx, &o->ls);
    if (rc == OC_OK) rc = oc_linsys_set_type(o->ls, o->cfg.linearSolver);
    if (rc == OC_OK && o->cfg.timing)
        for (auto& e : o->ev) cudaEventCreate(&e);
    if (rc != OC_OK) {
        oc_optimizer_destroy(o);
        return rc;
    }
    *out = o;
    return OC_OK;
}

int oc_optimizer_destroy(oc_optimizer* o)
{
    if (!o) return OC_ERR_INVALID;
    if (o->mesh && o->mesh->scafOwner == o) o->mesh->scafOwner = nullptr;
    cudaFree(o->g); cudaFree(o->dir); cudaFree(o->uv0);
    cudaFree(o->wuv); cudaFree(o->airCorner); cudaFree(o->airHb);
    o->air.uv = nullptr;
    device_mesh_free(o->air);
    if (o->ls) oc_linsys_destroy(o->ls);
    for (auto& e : o->ev)
        if (e) cudaEventDestroy(e);
    delete o;
    return OC_OK;
}

static void update_target_gres(oc_optimizer* o)
{
    // Optimizer::updateTargetGRes (Optimizer.cpp:675-678)
    // data0 is the mesh the Optimizer was constructed with: topology
    // operations on `result` leave this target unchanged
    o->targetGRes = o->param * static_cast<double>(o->nV0 - o->nFixed0) / static_cast<double>(o->nV0) * o->relGL2Tol;
}

// the mesh as the optimizer's kernels see it: with a scaffold, its UV is the
// leading part of the augmented UV
static oc::DeviceMesh mesh_view(const oc_optimizer* o)
{
    oc::DeviceMesh md = o->mesh->d;
    if (o->scaf) md.uv = o->wuv;
    return md;
}

static const double2* current_uv(const oc_optimizer* o) { return o->scaf ? o->wuv : o->mesh->d.uv; }

// Optimizer::computeEnergyVal (Optimizer.cpp:764-781) at uv + alphas[k] dir:
// energyParams[0] E_SD, plus with a scaffold w_scaf / |F_air| times the air
// mesh's uniform-weight E_SD (scafOut receives that part).
static int compute_energy(oc_optimizer* o, const double2* uv, const double2* dir, const double* alphas, int n,
                          double* out, double* scafOut = nullptr)
{
    oc_mesh* m = o->mesh;
    cudaStream_t st = m->ctx->stream;
    oc::launch_energy(mesh_view(o), uv, dir, alphas, n, 0, 1.0, m->scratch, st);
    o->launches += 2;
    if (o->scaf) {
        oc::launch_energy(o->air, uv, dir, alphas, n, 1, 1.0, m->scratch, st, m->scratch.result + oc::kMaxTrials);
        o->launches += 2;
    }
    double e[2 * oc::kMaxTrials];
    int rc = read_result(m, o->scaf ? 2 * oc::kMaxTrials : n, e);
    if (rc) return rc;
    for (int k = 0; k < n; ++k) {
        out[k] = o->param * e[k];   // Optimizer.cpp:767
        double es = 0.0;
        if (o->scaf) {
            es = e[oc::kMaxTrials + k] * o->airScale;   // Optimizer.cpp:776
            out[k] += es;
        }
        if (scafOut) scafOut[k] = es;
    }
    return OC_OK;
}

// (Re)builds the Newton-matrix pattern and its symbolic factorisation for
// the current system: the mesh alone, or mesh + air mesh in the augmented
// numbering (Scaffold::mergeVNeighbor / mergeFixedV, Scaffold.cpp:295-313,
// then LinSysSolver::set_pattern + analyze_pattern, Optimizer.cpp:521-527).
//
// A small scaffold (boundary + air vertices <= kCliqueMax) is given a
// pattern that does not depend on the air mesh's connectivity: every pair
// of boundary and air slots is a block (a clique, eliminated last as one
// dense front), with capAir >= the air-only vertex count padded by unused,
// decoupled slots.  Rebuilding the air mesh then changes only the values
// and the air contribution lists, not the analysis, as long as the
// boundary and capAir stay the same.  A larger scaffold gets the exact
// pattern, analysed again whenever its connectivity changes (as the
// reference re-analyses every iteration).
static constexpr int kCliqueMax = 512;

// The dissection tree of the solver's last analysis carried through the
// topology operations applied since (false: analyse from scratch).
static bool carried_tree(oc_optimizer* o, int nSys, const std::vector<int>* clique, std::vector<oc::NdNode>& out,
                         int& root)
{
    oc_mesh* m = o->mesh;
    oc_linsys* ls = o->ls;
    if (!o->cfg.carryAnalysis || ls->kind != OC_SOLVER_DIRECT || ls->analyzedVersion == ~0ULL ||
        ls->analyzedVersion > m->topoVersion)
        return false;
    std::vector<std::array<long long, 5>> edits;
    for (const auto& e : m->editLog)
        if (static_cast<unsigned long long>(e[0]) > ls->analyzedVersion) edits.push_back(e);
    if (edits.size() != m->topoVersion - ls->analyzedVersion) return false;
    for (size_t i = 0; i < edits.size(); ++i)
        if (static_cast<unsigned long long>(edits[i][0]) != ls->analyzedVersion + 1 + i) return false;
    auto t = std::chrono::steady_clock::now();
    const bool ok = carry_dissection(ls->chol, ls->analyzedMeshNV, edits, m->d.nV, nSys, clique, out, root);
    ls->carryMs = ms_since(t);
    return ok;
}

static int ensure_pattern(oc_optimizer* o)
{
    oc_mesh* m = o->mesh;
    const int nV = m->d.nV;
    if (o->patternStale) {
        int rc;
        std::vector<oc::NdNode> carried;
        int carriedRoot = -1;
        // current positions of the system's vertices: the ordering's
        // geometric bisection reads them
        const int nXY = o->cfg.ordering == OC_ORDER_BFS ? 0 : (o->scaf ? o->nWhole : nV);
        std::vector<double> xy(2 * (size_t)nXY);
        if (nXY) {
            OC_CUDA(m->ctx, cudaMemcpyAsync(xy.data(), o->scaf ? o->wuv : m->d.uv, sizeof(double2) * nXY,
                                            cudaMemcpyDeviceToHost, m->ctx->stream));
            OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
        }
        const double* xyp = nXY ? xy.data() : nullptr;
        if (!o->scaf) {
            std::vector<unsigned char> mask(nV, 0);
            for (int v : m->fixed) mask[v] = 1;
            const bool carry = carried_tree(o, nV, nullptr, carried, carriedRoot);
            rc = linsys_set_pattern(o->ls, nV, m->F.data(), m->d.nF, mask, nullptr, 0, nullptr, xyp, nullptr,
                                    nullptr, nullptr, carry ? &carried : nullptr, carriedRoot);
        }
        else {
            // rowFixed: 1 = fixed mesh vertex or unused air slot, 2 = fixed in
            // the air mesh as well (its diagonal also receives w_scaf / |F_air|)
            std::vector<unsigned char> mask(o->nWhole, 0);
            for (int v : m->fixed) mask[v] = 1;
            for (int v : m->fixed)
                for (int i = 0; i < o->nBnd; ++i)
                    if (o->bnd[i] == v) mask[v] = 2;
            for (int v = o->nWholeReal; v < o->nWhole; ++v) mask[v] = 1;
            if (o->cliqueMode) {
                // every air slot keeps its clique rows in the pattern, so that
                // a later air mesh with more air vertices fits it; the slots
                // this air mesh leaves unused are assembled as fixed rows
                std::vector<int> clique(o->bnd);
                for (int v = nV; v < o->nWhole; ++v) clique.push_back(v);
                std::vector<unsigned char> pmask(mask);
                for (int v = o->nWholeReal; v < o->nWhole; ++v) pmask[v] = 0;
                const bool carry = carried_tree(o, o->nWhole, &clique, carried, carriedRoot);
                rc = linsys_set_pattern(o->ls, o->nWhole, m->F.data(), m->d.nF, pmask, nullptr, 0, &clique, xyp,
                                        &mask, nullptr, nullptr, carry ? &carried : nullptr, carriedRoot);
            }
            else {
                // the exact air pattern (a scaffold too large for the clique):
                // with carried analyses the air-only vertices form the root
                // front above the mesh's dissection, a valid elimination tree
                // for every air mesh of the same boundary (each path through
                // the air crosses the root), so a rebuilt air mesh or a
                // topology operation re-derives only the front structures
                std::vector<int> airRoot;
                if (o->cfg.carryAnalysis)
                    for (int v = nV; v < o->nWhole; ++v) airRoot.push_back(v);
                const std::vector<int>* root = airRoot.empty() ? nullptr : &airRoot;
                const bool carry = root && carried_tree(o, o->nWhole, root, carried, carriedRoot);
                rc = linsys_set_pattern(o->ls, o->nWhole, m->F.data(), m->d.nF, mask, o->airFw.data(),
                                        static_cast<int>(o->airFw.size() / 3), nullptr, xyp, nullptr, nullptr,
                                        nullptr, carry ? &carried : nullptr, carriedRoot, root);
            }
        }
        if (rc) {
            o->ls->analyzedVersion = ~0ULL;
            return rc;
        }
        o->ls->analyzedVersion = m->topoVersion;
        o->ls->analyzedMeshNV = nV;
        o->patternStale = false;
        o->airContribStale = o->scaf;
    }
    if (o->scaf && o->airContribStale) {
        oc_linsys* ls = o->ls;
        std::vector<int> aPtr, aIdx;
        if (!air_contributions(ls->rowPtr, ls->col, ls->rowFixed, o->airFw.data(), static_cast<int>(o->airFw.size() / 3),
                               aPtr, aIdx))
            return fail(m->ctx, OC_ERR_INVALID, "scaffold: air triangle outside the pattern");
        cudaFree(ls->b.aPtr);
        cudaFree(ls->b.aIdx);
        ls->b.aPtr = ls->b.aIdx = nullptr;
        cudaStream_t st = m->ctx->stream;
        OC_CUDA(m->ctx, dalloc(&ls->b.aPtr, aPtr.size()));
        OC_CUDA(m->ctx, dalloc(&ls->b.aIdx, aIdx.size()));
        OC_CUDA(m->ctx, upload(ls->b.aPtr, aPtr.data(), aPtr.size(), st));
        OC_CUDA(m->ctx, upload(ls->b.aIdx, aIdx.data(), aIdx.size(), st));
        OC_CUDA(m->ctx, cudaStreamSynchronize(st));
        o->airContribStale = false;
    }
    return OC_OK;
}

// capacity of the augmented vectors (gradient, direction, UV copies)
static int ensure_whole(oc_optimizer* o, int n)
{
    if (n <= o->capWhole && o->wuv) return OC_OK;
    const int cap = std::max(n, o->capWhole);
    double2 *g = nullptr, *d = nullptr, *u0 = nullptr, *w = nullptr;
    if (dalloc(&g, cap) != cudaSuccess || dalloc(&d, cap) != cudaSuccess || dalloc(&u0, cap) != cudaSuccess ||
        dalloc(&w, cap) != cudaSuccess) {
        cudaFree(g); cudaFree(d); cudaFree(u0); cudaFree(w);
        return fail(o->mesh->ctx, OC_ERR_CUDA, "optimizer: augmented vector alloc");
    }
    cudaFree(o->g); cudaFree(o->dir); cudaFree(o->uv0); cudaFree(o->wuv);
    o->g = g; o->dir = d; o->uv0 = u0; o->wuv = w;
    o->capWhole = cap;
    return OC_OK;
}

int oc_optimizer_precompute(oc_optimizer* o)
{
    if (!o) return OC_ERR_INVALID;
    oc_mesh* m = o->mesh;
    int ok = 0;
    int rc = oc_mesh_check_inversion(m, &ok);   // Optimizer.cpp:65-67
    if (rc) return rc;
    if (!ok) return fail(m->ctx, OC_ERR_INVERTED, "precompute: inverted UV triangle");
    o->patternStale = true;
    rc = ensure_pattern(o);
    if (rc) return rc;
    if (o->scaf)
        OC_CUDA(m->ctx, cudaMemcpyAsync(o->wuv, m->d.uv, sizeof(double2) * m->d.nV, cudaMemcpyDeviceToDevice,
                                        m->ctx->stream));
    o->lastEDec = 0.0;
    update_target_gres(o);
    rc = compute_energy(o, current_uv(o), nullptr, nullptr, 1, &o->lastEnergyVal, &o->eScaf);
    if (rc) return rc;
    o->precomputed = true;
    return OC_OK;
}

// One Newton iteration: Optimizer::solve's body (Optimizer.cpp:208-230) with
// solve_oneStep (:505-573) and lineSearch (:575-652), including the
// scaffolding branches when an air mesh is set.
static int solve_one(oc_optimizer* o, int* converged)
{
    oc_mesh* m = o->mesh;
    oc_ctx* ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    const oc::DeviceMesh md = mesh_view(o);
    const int nSys = o->scaf ? o->nWhole : m->d.nV;
    *converged = 0;
    record(o, 0);
    if (o->scaf) {
        oc::launch_gradient_scaf(md, o->param, m->cornerBuf, o->air, o->airScale, o->airCorner, o->g, m->scratch, st);
        o->launches += 4;
    }
    else {
        oc::launch_gradient(md, 0, o->param, m->cornerBuf, o->g, m->scratch, st);
        o->launches += 3;
    }
    double gsq = 0.0;
    int rc = read_result(m, 1, &gsq);
    if (rc) return rc;
    o->lastGsq = gsq;
    record(o, 1);
    if (gsq < o->targetGRes) {
        o->lastEDec = 0.0;
        o->globalIterNum++;
        o->lastStep = 0.0;
        o->lastPcgIters = 0;
        o->lastLsLaunches = 0;
        *converged = 1;
        if (o->cfg.timing) {
            cudaEventSynchronize(o->ev[1]);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, o->ev[0], o->ev[1]);
            o->phaseMs[0] += ms;
        }
        return OC_OK;
    }
    // Hessian + PSD projection (computeHessian), block assembly (update_a)
    oc::launch_hessian(md, 0, m->hb, st, o->cfg.hessianProjection);
    if (o->scaf) oc::launch_hessian(o->air, 1, o->airHb, st, o->cfg.hessianProjection);
    record(o, 2);
    if (o->scaf) oc::launch_assemble_scaf(o->ls->b, m->hb, m->d.nF, o->param, o->airHb, o->air.nF, o->airScale, st);
    else oc::launch_assemble(o->ls->b, m->hb, m->d.nF, o->param, st);
    o->launches += o->scaf ? 3 : 2;
    record(o, 3);
    // factorize (direct) or block-Jacobi preconditioner (PCG); fixed rows =
    // param * I (+ w_scaf / |F_air| * I when also fixed in the air mesh)
    int bad = 0;
    rc = linsys_factor(o->ls, o->param, &bad, o->param + o->airScale);
    if (rc) return rc;
    o->badPivots = bad;
    o->launches += 1 + (o->ls->kind == OC_SOLVER_DIRECT ? 3 + (long long)o->ls->chol.launches.size() : 0);
    if (bad > 0)   // Optimizer.cpp:548-554 dumps the matrix and exits
        return fail(ctx, OC_ERR_NOT_SPD,
                    "solve: " + std::to_string(bad) + " zero or non-finite pivot(s) in the Newton matrix");
    record(o, 4);
    // search direction: H d = -g
    std::string err;
    int iters = 0;
    double relres = 0.0;
    int solveStatus = OC_OK;
    if (o->ls->kind == OC_SOLVER_DIRECT) {
        rc = oc::chol_solve(o->ls->chol, o->g, o->dir, -1.0, st, &err);
        if (rc) return fail(ctx, rc, err);
        o->launches += 2 + 2LL * o->ls->chol.nLevels;
    }
    else {
        rc = oc::pcg_solve(o->ls->b, o->g, o->dir, o->ls->wk, o->cfg.pcgTol, o->cfg.pcgMaxIter, -1.0, st, &iters,
                           &relres, &err);
        o->launches += 1;
        if (rc == OC_ERR_CUDA) return fail(ctx, rc, err);
        solveStatus = rc;
    }
    o->lastPcgIters = iters;
    o->lastRelRes = relres;
    record(o, 5);
    // Optimizer::lineSearch: injective bound over the mesh and the air mesh
    // (Optimizer::initStepSize, :692-704), then halve until E <= E_last
    oc::launch_init_step(md, o->dir, 1.0, m->scratch, st);
    o->launches += 2;
    if (o->scaf) {
        oc::launch_init_step(o->air, o->dir, 1.0, m->scratch, st, false);
        o->launches += 1;
    }
    double step = 1.0;
    rc = read_min(m, &step);
    if (rc) return rc;
    if (o->ls->kind == OC_SOLVER_DIRECT) {   // the substitutions' bounded waits
        int timedOut = 0;
        rc = oc::chol_solve_status(o->ls->chol, st, &timedOut);
        if (rc) return fail(ctx, rc, "solve: substitution status");
        if (timedOut) return fail(ctx, OC_ERR_TIMEOUT, "solve: a substitution wait ran out");
    }
    record(o, 6);
    step *= 0.99;
    OC_CUDA(ctx, cudaMemcpyAsync(o->uv0, current_uv(o), sizeof(double2) * nSys, cudaMemcpyDeviceToDevice, st));
    bool stopped = false;
    double testE = 0.0, testScaf = 0.0, accepted = -1.0, lastTried = step, lastTriedE = 0.0, lastTriedScaf = 0.0;
    double lastScaf0 = 0.0;
    int lsLaunches = 0;
    int batch = 1;
    double alpha = step;
    bool first = true;
    while (accepted < 0.0) {
        double alphas[oc::kMaxTrials], E[oc::kMaxTrials], Es[oc::kMaxTrials];
        int n = 0;
        // with a scaffold the first launch also re-evaluates E at the current
        // point (alpha = 0): lastEnergyVal is recomputed because the air
        // mesh changed since the last step (Optimizer.cpp:588-592)
        const int lead = (first && o->scaf) ? 1 : 0;
        if (lead) alphas[n++] = 0.0;
        for (double a = alpha; n < batch + lead && a != 0.0; a /= 2.0) alphas[n++] = a;
        if (n == lead) break;
        rc = compute_energy(o, o->uv0, o->dir, alphas, n, E, Es);
        if (rc) return rc;
        ++lsLaunches;
        if (lead) {
            o->lastEnergyVal = E[0];
            lastScaf0 = Es[0];
        }
        for (int k = lead; k < n; ++k) {
            lastTried = alphas[k];
            lastTriedE = E[k];
            lastTriedScaf = Es[k];
            if (!(E[k] > o->lastEnergyVal)) {   // while(testingE > lastEnergyVal) halves, Optimizer.cpp:597
                accepted = alphas[k];
                testE = E[k];
                testScaf = Es[k];
                break;
            }
        }
        alpha = alphas[n - 1] / 2.0;
        batch = o->cfg.lineSearchBatch;
        first = false;
    }
    if (accepted < 0.0) {   // step reached 0 (Optimizer.cpp:600-606): keep the last trial
        stopped = true;
        accepted = lastTried;
        testE = lastTriedE;
        testScaf = lastTriedScaf;
    }
    if (o->scaf) {
        oc::launch_step_forward(o->uv0, o->dir, accepted, o->wuv, nSys, st);
        OC_CUDA(ctx, cudaMemcpyAsync(m->d.uv, o->wuv, sizeof(double2) * m->d.nV, cudaMemcpyDeviceToDevice, st));
    }
    else {
        oc::launch_step_forward(o->uv0, o->dir, accepted, m->d.uv, nSys, st);
    }
    o->launches += 1;
    OC_CUDA(ctx, cudaGetLastError());
    record(o, 7);
    o->lastEDec = o->lastEnergyVal - testE;
    if (o->scaf) o->lastEDec += (-lastScaf0 + testScaf);   // Optimizer.cpp:632-634
    if (o->allowEDecRelTol && (o->lastEDec / o->lastEnergyVal < 1.0e-6 * accepted) && (accepted > 1.0e-3))
        stopped = true;   // :635-638
    o->lastEnergyVal = testE;
    o->eScaf = testScaf;
    o->lastStep = accepted;
    o->lastLsLaunches = lsLaunches;
    o->globalIterNum++;
    if (o->cfg.timing) {
        cudaEventSynchronize(o->ev[7]);
        for (int k = 0; k < 7; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, o->ev[k], o->ev[k + 1]);
            o->phaseMs[k] += ms;
        }
    }
    *converged = stopped ? 1 : 0;
    return solveStatus == OC_ERR_NOT_CONVERGED ? OC_ERR_NOT_CONVERGED : OC_OK;
}

int oc_optimizer_solve(oc_optimizer* o, int maxIter, int* result)
{
    if (!o || !result || maxIter < 0) return OC_ERR_INVALID;
    if (!o->precomputed) return fail(o->mesh->ctx, OC_ERR_INVALID, "solve before precompute");
    *result = 0;
    int status = OC_OK;
    int prc = ensure_pattern(o);
    if (prc) return prc;
    if (o->scaf)   // the mesh's UV is authoritative (oc_mesh_set_uv may have moved it)
        OC_CUDA(o->mesh->ctx, cudaMemcpyAsync(o->wuv, o->mesh->d.uv, sizeof(double2) * o->mesh->d.nV,
                                              cudaMemcpyDeviceToDevice, o->mesh->ctx->stream));
    for (int it = 0; it < maxIter; ++it) {
        int conv = 0;
        int rc = solve_one(o, &conv);
        if (rc != OC_OK && rc != OC_ERR_NOT_CONVERGED) return rc;
        if (rc == OC_ERR_NOT_CONVERGED) status = rc;
        if (conv) {
            *result = 1;
            return status;
        }
    }
    return status;
}

int oc_optimizer_get_last_energy(oc_optimizer* o, double* e)
{
    if (!o || !e) return OC_ERR_INVALID;
    *e = o->lastEnergyVal;
    return OC_OK;
}

int oc_optimizer_get_iter_num(oc_optimizer* o, int* n)
{
    if (!o || !n) return OC_ERR_INVALID;
    *n = o->globalIterNum;
    return OC_OK;
}

int oc_optimizer_set_rel_gl2_tol(oc_optimizer* o, double tol)
{
    if (!o || !(tol > 0.0)) return OC_ERR_INVALID;
    o->relGL2Tol = tol;
    update_target_gres(o);
    return OC_OK;
}

int oc_optimizer_set_energy_param(oc_optimizer* o, double p)
{
    if (!o || !(p > 0.0)) return OC_ERR_INVALID;
    o->param = p;
    update_target_gres(o);
    if (!o->precomputed) return OC_OK;
    if (o->scaf)
        OC_CUDA(o->mesh->ctx, cudaMemcpyAsync(o->wuv, o->mesh->d.uv, sizeof(double2) * o->mesh->d.nV,
                                              cudaMemcpyDeviceToDevice, o->mesh->ctx->stream));
    return compute_energy(o, current_uv(o), nullptr, nullptr, 1, &o->lastEnergyVal, &o->eScaf);
}

int oc_optimizer_last_step(oc_optimizer* o, double* stepSize, int* pcgIters, double* pcgRelRes, int* lsLaunches,
                           double* gsq)
{
    if (!o) return OC_ERR_INVALID;
    if (stepSize) *stepSize = o->lastStep;
    if (pcgIters) *pcgIters = o->lastPcgIters;
    if (pcgRelRes) *pcgRelRes = o->lastRelRes;
    if (lsLaunches) *lsLaunches = o->lastLsLaunches;
    if (gsq) *gsq = o->lastGsq;
    return OC_OK;
}

int oc_optimizer_last_edec(oc_optimizer* o, double* eDec)
{
    if (!o || !eDec) return OC_ERR_INVALID;
    *eDec = o->lastEDec;
    return OC_OK;
}

int oc_optimizer_set_allow_edec_rel_tol(oc_optimizer* o, int allow)
{
    if (!o) return OC_ERR_INVALID;
    o->allowEDecRelTol = allow != 0;
    return OC_OK;
}

int oc_optimizer_get_energy_param(oc_optimizer* o, double* energyParam)
{
    if (!o || !energyParam) return OC_ERR_INVALID;
    *energyParam = o->param;
    return OC_OK;
}

int oc_optimizer_set_state(oc_optimizer* o, int nV, const double* Vrest, const double* UV, int nF, const int* F,
                           int nCohE, const int* cohE, const int* tails3, int iterNum)
{
    // Optimizer::setConfig (Optimizer.cpp:287-300): the result mesh replaced
    // by a recorded one, the scaffold rebuilt, the energy data updated
    if (!o || !o->precomputed || nV <= 0 || nF <= 0 || nCohE < 0 || !Vrest || !UV || !F || (nCohE && !cohE) ||
        iterNum < 0)
        return OC_ERR_INVALID;
    oc_mesh* m = o->mesh;
    // topology operations keep the triangle count (splits and merges move
    // corners between vertices), so a recorded state of this run has it too
    if (nF != m->d.nF) return fail(m->ctx, OC_ERR_INVALID, "set_state: triangle count differs from the mesh's");
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return fail(m->ctx, OC_ERR_INVALID, "set_state: vertex index out of range");
    for (long long i = 0; i < 4LL * nCohE; ++i)
        if (cohE[i] < -1 || cohE[i] >= nV) return fail(m->ctx, OC_ERR_INVALID, "set_state: cohesive edge out of range");
    for (int v : m->fixed)
        if (v >= nV) return fail(m->ctx, OC_ERR_INVALID, "set_state: fixed vertex out of range");
    if (tails3)
        for (int k = 0; k < 3; ++k)
            if (tails3[k] < -1 || tails3[k] >= nV) return fail(m->ctx, OC_ERR_INVALID, "set_state: tail out of range");
    m->F.assign(F, F + 3 * (size_t)nF);
    m->Vrest.assign(Vrest, Vrest + 3 * (size_t)nV);
    m->cohE.assign(cohE, cohE + 4 * (size_t)nCohE);
    if (tails3) std::copy(tails3, tails3 + 3, m->tails);
    std::vector<double> uv(UV, UV + 2 * (size_t)nV);
    int rc = mesh_rebuild(m, uv);
    if (rc) return rc;
    rc = ensure_whole(o, nV);
    if (rc) return rc;
    if (!o->scaf) o->nWhole = o->nWholeReal = nV;
    o->patternStale = true;
    if (o->scaf) {
        rc = oc_optimizer_rebuild_scaffold(o);
        if (rc) return rc;
    }
    rc = ensure_pattern(o);
    if (rc) return rc;
    if (o->scaf)
        OC_CUDA(m->ctx, cudaMemcpyAsync(o->wuv, m->d.uv, sizeof(double2) * nV, cudaMemcpyDeviceToDevice, m->ctx->stream));
    o->globalIterNum = iterNum;
    update_target_gres(o);
    return compute_energy(o, current_uv(o), nullptr, nullptr, 1, &o->lastEnergyVal, &o->eScaf);
}

int oc_optimizer_bad_pivots(oc_optimizer* o, int* nBad)
{
    if (!o || !nBad) return OC_ERR_INVALID;
    *nBad = o->badPivots;
    return OC_OK;
}

int oc_optimizer_phase_ms(oc_optimizer* o, double* out7)
{
    if (!o || !out7) return OC_ERR_INVALID;
    for (int k = 0; k < 7; ++k) {
        out7[k] = o->phaseMs[k];
        o->phaseMs[k] = 0.0;
    }
    return OC_OK;
}

int oc_optimizer_solver_stats(oc_optimizer* o, double* out8)
{
    if (!o) return OC_ERR_INVALID;
    return oc_linsys_stats(o->ls, out8);
}

int oc_optimizer_set_solve_cluster(oc_optimizer* o, int maxCluster)
{
    if (!o) return OC_ERR_INVALID;
    return oc_linsys_set_solve_cluster(o->ls, maxCluster);
}

int oc_optimizer_solve_clusters(oc_optimizer* o, int* levels, int* largest)
{
    if (!o) return OC_ERR_INVALID;
    return oc_linsys_solve_clusters(o->ls, levels, largest);
}

int oc_optimizer_set_factor_streams(oc_optimizer* o, int streams)
{
    if (!o) return OC_ERR_INVALID;
    return oc_linsys_set_factor_streams(o->ls, streams);
}

int oc_optimizer_factor_streams(oc_optimizer* o, int* streams, int* groups)
{
    if (!o) return OC_ERR_INVALID;
    return oc_linsys_factor_streams(o->ls, streams, groups);
}

int oc_optimizer_set_scaffold(oc_optimizer* o, const double* airV, int nAirV, const int* airF, int nAirF,
                              const int* bnd, int nBnd, double areaThres)
{
    if (!o || !airV || !airF || !bnd || nAirF <= 0 || nBnd <= 0 || nAirV < nBnd) return OC_ERR_INVALID;
    oc_mesh* m = o->mesh;
    oc_ctx* ctx = m->ctx;
    const int nV = m->d.nV;
    if ((long long)nV + nAirV - nBnd >= (1LL << 30) || ((long long)m->d.nF + nAirF) * 9 >= (1LL << 31))
        return fail(ctx, OC_ERR_INVALID, "set_scaffold: system too large");
    for (long long i = 0; i < 3LL * nAirF; ++i)
        if (airF[i] < 0 || airF[i] >= nAirV) return fail(ctx, OC_ERR_INVALID, "set_scaffold: air vertex index out of range");
    std::vector<int> isBnd(nV, -1);
    for (int i = 0; i < nBnd; ++i) {
        if (bnd[i] < 0 || bnd[i] >= nV) return fail(ctx, OC_ERR_INVALID, "set_scaffold: boundary vertex out of range");
        if (isBnd[bnd[i]] >= 0) return fail(ctx, OC_ERR_INVALID, "set_scaffold: repeated boundary vertex");
        isBnd[bnd[i]] = i;
    }
    // areaThres_AM = sqrt(3)/4 edgeLen_eps^2, edgeLen_eps = avgEdgeLen / 2
    // for a whole-mesh scaffold (Scaffold.cpp:34, 189)
    if (!(areaThres >= 0.0)) {
        const double eps = m->scalars[1] * 0.5;
        areaThres = std::sqrt(3.0) / 4.0 * eps * eps;
    }
    // air mesh rest shape = its own layout, z = 0 (Scaffold.cpp:187-190)
    std::vector<double> V3(3 * (size_t)nAirV);
    for (int i = 0; i < nAirV; ++i) {
        V3[3 * (size_t)i] = airV[2 * (size_t)i];
        V3[3 * (size_t)i + 1] = airV[2 * (size_t)i + 1];
        V3[3 * (size_t)i + 2] = 0.0;
    }
    std::vector<double> rest;
    double area = 0.0;
    if (!rest_constants(V3.data(), airF, nAirF, areaThres, rest, area))
        return fail(ctx, OC_ERR_DEGENERATE, "set_scaffold: zero-area air triangle");
    const int nAirOnly = nAirV - nBnd;
    // clique pattern for small scaffolds: air slots padded to a multiple of
    // 32, reused while the air-only count fits and the boundary is unchanged
    int capAir = (nAirOnly + 31) / 32 * 32;
    // the same boundary vertex set (the clique does not depend on their order)
    bool sameBnd = false;
    if (o->scaf && (int)o->bnd.size() == nBnd) {
        std::vector<int> x(bnd, bnd + nBnd), y(o->bnd);
        std::sort(x.begin(), x.end());
        std::sort(y.begin(), y.end());
        sameBnd = x == y;
    }
    if (sameBnd && o->cliqueMode && nAirOnly <= o->capAir && o->capAir - nAirOnly <= 64) capAir = o->capAir;
    const bool cliqueMode = o->cfg.scaffoldPattern == 0 && nBnd + capAir <= kCliqueMax;
    if (!cliqueMode) capAir = nAirOnly;
    const int nWhole = nV + capAir;
    auto toWhole = [&](int a) { return a < nBnd ? bnd[a] : nV + a - nBnd; };   // localVI2Global
    std::vector<int> Fw(3 * (size_t)nAirF);
    for (size_t i = 0; i < Fw.size(); ++i) Fw[i] = toWhole(airF[i]);
    // fixed air vertices: the mesh's fixed vertices on the boundary (Scaffold.cpp:193-199)
    std::vector<unsigned char> airMask(nWhole, 0);
    for (int v : m->fixed)
        if (isBnd[v] >= 0) airMask[v] = 1;
    const bool samePattern = o->scaf && !o->patternStale && sameBnd && o->nWhole == nWhole &&
                             o->cliqueMode == cliqueMode &&
                             (cliqueMode || (Fw == o->airFw && std::equal(bnd, bnd + nBnd, o->bnd.begin())));
    int rc = ensure_whole(o, nWhole);
    if (rc) return rc;
    if (nAirF > o->capAirF) {
        cudaFree(o->airCorner); cudaFree(o->airHb);
        o->airCorner = nullptr; o->airHb = nullptr;
        o->capAirF = 0;
        if (dalloc(&o->airCorner, 3 * (size_t)nAirF) != cudaSuccess || dalloc(&o->airHb, 21 * (size_t)nAirF) != cudaSuccess)
            return fail(ctx, OC_ERR_CUDA, "set_scaffold: alloc");
        o->capAirF = nAirF;
    }
    o->air.uv = nullptr;
    rc = device_mesh_upload(ctx, o->air, nWhole, Fw.data(), nAirF, rest, area, airMask);
    if (rc) return rc;
    o->air.uv = o->wuv;
    cudaStream_t st = ctx->stream;
    OC_CUDA(ctx, cudaMemcpyAsync(o->wuv, m->d.uv, sizeof(double2) * nV, cudaMemcpyDeviceToDevice, st));
    if (nAirV > nBnd)
        OC_CUDA(ctx, cudaMemcpyAsync(o->wuv + nV, airV + 2 * (size_t)nBnd, sizeof(double2) * (nAirV - nBnd),
                                     cudaMemcpyHostToDevice, st));
    if (nWhole > nV + nAirOnly)   // unused air slots: not in any triangle, kept at 0
        OC_CUDA(ctx, cudaMemsetAsync(o->wuv + nV + nAirOnly, 0, sizeof(double2) * (nWhole - nV - nAirOnly), st));
    OC_CUDA(ctx, cudaStreamSynchronize(st));
    o->airFw.swap(Fw);
    o->airF.assign(airF, airF + 3 * (size_t)nAirF);
    o->bnd.assign(bnd, bnd + nBnd);
    o->nWhole = nWhole;
    o->nWholeReal = nV + nAirOnly;
    o->capAir = capAir;
    o->cliqueMode = cliqueMode;
    o->nAirV = nAirV;
    o->nBnd = nBnd;
    o->airScale = o->wScaf / nAirF;   // w_scaf / airMesh.F.rows() (Optimizer.cpp:776)
    o->scaf = true;
    m->scafOwner = o;   // result.scaffold = &scaffold
    if (!samePattern) o->patternStale = true;
    else if (cliqueMode) {
        // the kept pattern's padding may now cover slots the previous air mesh
        // used (or the reverse): unused slots are fixed rows, so that their
        // decoupled diagonal blocks hold param * I instead of zero
        oc_linsys* ls = o->ls;
        bool changed = false;
        for (int v = nV; v < nWhole; ++v) {
            const unsigned char f = v >= nV + nAirOnly ? 1 : 0;
            if (ls->rowFixed[v] != f) {
                ls->rowFixed[v] = f;
                changed = true;
            }
        }
        if (changed)
            OC_CUDA(ctx, cudaMemcpyAsync(ls->b.rowFixed + nV, ls->rowFixed.data() + nV, nWhole - nV,
                                         cudaMemcpyHostToDevice, st));
    }
    o->airContribStale = true;
    return OC_OK;
}

int oc_optimizer_create_fracture(oc_optimizer* o, int opType, const int* path, int pathLen, const double* newVertPos,
                                 int posRows)
{
    // Optimizer::createFracture(opType, path, newVertPos, ...) (Optimizer.cpp:373-440)
    if (!o || !o->precomputed) return OC_ERR_INVALID;
    oc_mesh* m = o->mesh;
    std::fill(o->applyMs, o->applyMs + 6, 0.0);
    int rc = apply_topology(m, opType, path, pathLen, newVertPos, posRows, o->applyMs);
    if (rc) return rc;
    auto t = std::chrono::steady_clock::now();
    const int nV = m->d.nV;
    rc = ensure_whole(o, nV);
    if (rc) return rc;
    if (!o->scaf) o->nWhole = o->nWholeReal = nV;
    o->patternStale = true;
    if (o->scaf) {   // scaffold = Scaffold(result, ...) (:416-421)
        rc = oc_optimizer_rebuild_scaffold(o);
        if (rc) return rc;
    }
    o->applyMs[2] = ms_since(t);
    o->ls->patternHostMs = o->ls->patternDevMs = 0.0;
    rc = ensure_pattern(o);   // updateEnergyData(true, false, true) (:423-425)
    if (rc) return rc;
    ms_since(t);
    o->applyMs[3] = o->ls->patternHostMs;
    o->applyMs[4] = o->ls->patternDevMs;
    if (o->scaf)
        OC_CUDA(m->ctx, cudaMemcpyAsync(o->wuv, m->d.uv, sizeof(double2) * nV, cudaMemcpyDeviceToDevice, m->ctx->stream));
    rc = compute_energy(o, current_uv(o), nullptr, nullptr, 1, &o->lastEnergyVal, &o->eScaf);
    o->applyMs[5] = ms_since(t);
    return rc;
}

int oc_optimizer_analysis_info(oc_optimizer* o, int* carried, double* ndMs, double* symMs, double* flops,
                               double* fullFlops)
{
    if (!o || !o->ls) return OC_ERR_INVALID;
    const oc::CholPlan& P = o->ls->chol;
    if (carried) *carried = P.incremental;
    if (ndMs) *ndMs = P.ndMs;
    if (symMs) *symMs = P.symMs;
    if (flops) *flops = P.flops;
    if (fullFlops) *fullFlops = P.fullFlops;
    return OC_OK;
}

int oc_optimizer_apply_timing(oc_optimizer* o, double* out6)
{
    if (!o || !out6) return OC_ERR_INVALID;
    std::copy(o->applyMs, o->applyMs + 6, out6);
    return OC_OK;
}

int oc_optimizer_split_or_merge(oc_optimizer* o, double EDecThres, int splitInterior, double filterExp, int options,
                                oc_mlp* mlp, double topFrac, int* changed, int* opType, double* EwDecMax)
{
    // Optimizer::createFracture(stressThres, 0, false, allowInSplit)
    // (Optimizer.cpp:440-503) -> TriMesh::splitOrMerge (TriMesh.cpp:978-1052)
    if (!o || !o->precomputed || !changed) return OC_ERR_INVALID;
    *changed = 0;
    oc_mesh* m = o->mesh;
    const double lambda_t = 1.0 - o->param;
    auto run = [&](int op, oc_topo_result** r) {
        return mlp ? oc_topology_query_learned(m, op, lambda_t, filterExp, options, mlp, topFrac, r)
                   : oc_topology_query(m, op, lambda_t, filterExp, options, r);
    };
    auto bestOf = [](const oc_topo_result* r) { return r->best >= 0 ? r->cands[r->best].EwDec : -DBL_MAX; };
    oc_topo_result *a = nullptr, *b = nullptr;
    int rc = run(splitInterior ? oc::kOpInteriorSplit : oc::kOpBoundarySplit, &a);
    if (!rc && !splitInterior) rc = run(oc::kOpMerge, &b);
    if (rc) {
        oc_topo_result_destroy(a);
        oc_topo_result_destroy(b);
        return rc;
    }
    // the larger decrease of split and merge, split on ties (TriMesh.cpp:1002-1013)
    const oc_topo_result* pick = a;
    int op = splitInterior ? oc::kOpInteriorSplit : oc::kOpBoundarySplit;
    if (b && bestOf(b) > bestOf(a)) {
        pick = b;
        op = oc::kOpMerge;
    }
    const double best = bestOf(pick);
    if (opType) *opType = op;
    if (EwDecMax) *EwDecMax = best;
    if (best > EDecThres && pick->best >= 0) {   // TriMesh.cpp:1015
        const oc::TopoCandidate& C = pick->cands[pick->best];
        rc = oc_optimizer_create_fracture(o, op, C.path.data(), static_cast<int>(C.path.size()), C.pos.data(),
                                          static_cast<int>(C.pos.size() / 2));
        if (!rc) *changed = 1;
    }
    oc_topo_result_destroy(a);
    oc_topo_result_destroy(b);
    return rc;
}

int oc_optimizer_rebuild_scaffold(oc_optimizer* o)
{
    if (!o) return OC_ERR_INVALID;
    oc_mesh* m = o->mesh;
    std::vector<double> uv(2 * (size_t)m->d.nV);
    OC_CUDA(m->ctx, cudaMemcpyAsync(uv.data(), m->d.uv, sizeof(double2) * m->d.nV, cudaMemcpyDeviceToHost,
                                    m->ctx->stream));
    OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
    oc::AirMesh am;
    std::string err;
    if (o->bndVersion != m->topoVersion) {
        const int rb = oc::air_mesh_boundary(m->d.nV, m->F.data(), m->d.nF, o->bndLoops, o->bndLoopStart,
                                             o->bndSeeds, &err);
        if (rb) return fail(m->ctx, rb, err);
        o->bndVersion = m->topoVersion;
    }
    const int rc = oc::air_mesh_build_loops(uv.data(), m->d.nV, o->bndLoops, o->bndLoopStart, o->bndSeeds,
                                            m->scalars[1], am, &err);
    if (rc) return fail(m->ctx, rc, err);
    return oc_optimizer_set_scaffold(o, am.V.data(), static_cast<int>(am.V.size() / 2), am.F.data(),
                                     static_cast<int>(am.F.size() / 3), am.bnd.data(), am.nBnd, -1.0);
}

int oc_optimizer_clear_scaffold(oc_optimizer* o)
{
    if (!o) return OC_ERR_INVALID;
    if (o->scaf) o->patternStale = true;
    o->scaf = false;
    if (o->mesh && o->mesh->scafOwner == o) o->mesh->scafOwner = nullptr;
    o->eScaf = 0.0;
    o->nWhole = o->nWholeReal = o->mesh->d.nV;
    return OC_OK;
}

int oc_optimizer_get_scaffold(oc_optimizer* o, int* nAirV, int* nAirF, int* nBnd, double* airV, int* airF, int* bnd)
{
    if (!o || !o->scaf) return OC_ERR_INVALID;
    oc_mesh* m = o->mesh;
    if (nAirV) *nAirV = o->nAirV;
    if (nAirF) *nAirF = static_cast<int>(o->airF.size() / 3);
    if (nBnd) *nBnd = o->nBnd;
    if (airF) std::copy(o->airF.begin(), o->airF.end(), airF);
    if (bnd) std::copy(o->bnd.begin(), o->bnd.end(), bnd);
    if (airV) {
        std::vector<double> w(2 * (size_t)o->nWhole);
        OC_CUDA(m->ctx, cudaMemcpyAsync(w.data(), o->wuv, sizeof(double2) * o->nWhole, cudaMemcpyDeviceToHost,
                                        m->ctx->stream));
        OC_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
        for (int i = 0; i < o->nAirV; ++i) {
            const int v = i < o->nBnd ? o->bnd[i] : m->d.nV + i - o->nBnd;
            airV[2 * (size_t)i] = w[2 * (size_t)v];
            airV[2 * (size_t)i + 1] = w[2 * (size_t)v + 1];
        }
    }
    return OC_OK;
}

int oc_optimizer_get_last_energy_scaffold(oc_optimizer* o, double* eScaf)
{
    if (!o || !eScaf) return OC_ERR_INVALID;
    *eScaf = o->eScaf;
    return OC_OK;
}

int oc_optimizer_system_size(oc_optimizer* o, int* nVerts)
{
    if (!o || !nVerts) return OC_ERR_INVALID;
    *nVerts = o->scaf ? o->nWholeReal : o->mesh->d.nV;
    return OC_OK;
}

int oc_optimizer_last_vectors(oc_optimizer* o, double* gradient, double* searchDir)
{
    if (!o) return OC_ERR_INVALID;
    oc_mesh* m = o->mesh;
    const int n = o->scaf ? o->nWholeReal : m->d.nV;
    cudaStream_t st = m->ctx->stream;
    if (gradient) OC_CUDA(m->ctx, cudaMemcpyAsync(gradient, o->g, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    if (searchDir) OC_CUDA(m->ctx, cudaMemcpyAsync(searchDir, o->dir, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    OC_CUDA(m->ctx, cudaStreamSynchronize(st));
    return OC_OK;
}

int oc_optimizer_launch_count(oc_optimizer* o, long long* n)
{
    if (!o || !n) return OC_ERR_INVALID;
    *n = o->launches;
    return OC_OK;
}

} // extern "C"
