// Host side of the C ABI (include/optcuts_gpu.h): context, device mesh,
// linear solver and the projected-Newton Optimizer, each mirroring the
// reference class it replaces (TriMesh, SymDirichletEnergy, LinSysSolver /
// EigenLibSolver, Optimizer).  No exception crosses the ABI; every entry
// point returns an oc_status.

#include "oc_chol.h"
#include "oc_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

struct oc_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    int nsm = 0;
    std::string err;
};

struct oc_mesh {
    oc_ctx* ctx = nullptr;
    oc::DeviceMesh d;
    oc::Scratch scratch;
    std::vector<double> rest;       // nF x 8, TriMesh feature layout
    double scalars[3] = {0, 0, 0};  // surfaceArea, avgEdgeLen, virtualRadius
    std::vector<int> F, fixed;
    double2* cornerBuf = nullptr;   // 3 x nF corner gradients
    double2* tmpV = nullptr;        // nV scratch
    double* hb = nullptr;           // 21 x nF packed Hessians
    double* tmpF = nullptr;         // nF x 36 scratch for API outputs (lazy)
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
};

struct oc_optimizer {
    oc_mesh* mesh = nullptr;
    oc_linsys* ls = nullptr;
    oc_optimizer_config cfg;
    double param = 1.0, relGL2Tol = 1e-12, targetGRes = 0.0;
    double lastEnergyVal = 0.0, lastEDec = 0.0;
    int globalIterNum = 0;
    bool precomputed = false;
    double2 *g = nullptr, *dir = nullptr, *uv0 = nullptr;
    // last-step diagnostics
    double lastStep = 0.0, lastRelRes = 0.0, lastGsq = 0.0;
    int lastPcgIters = 0, lastLsLaunches = 0;
    long long launches = 0;
    int badPivots = 0;
    cudaEvent_t ev[9] = {};
    double phaseMs[7] = {0, 0, 0, 0, 0, 0, 0};
};

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

// Full-symmetric 2x2-block pattern from the triangles (the vertex adjacency
// LinSysSolver::set_pattern reads from TriMesh::vNeighbor,
// LinSysSolver.hpp:37-135).  Fixed rows keep only their diagonal block.
// Also produces, per block slot, the ordered list of triangle contributions
// (t * 9 + a * 3 + b), free-free pairs only.
void build_pattern(int nV, const int* F, int nF, const std::vector<unsigned char>& fixedMask,
                   std::vector<int>& rowPtr, std::vector<int>& col, std::vector<int>& diagSlot,
                   std::vector<int>& cPtr, std::vector<int>& cIdx)
{
    std::vector<int> deg(nV, 1);
    std::vector<std::vector<int>> nb(nV);
    for (int v = 0; v < nV; ++v) nb[v].push_back(v);
    for (int t = 0; t < nF; ++t)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                if (a == b) continue;
                const int va = F[3 * t + a], vb = F[3 * t + b];
                if (fixedMask[va] || fixedMask[vb]) continue;
                nb[va].push_back(vb);
            }
    rowPtr.assign(nV + 1, 0);
    for (int v = 0; v < nV; ++v) {
        std::sort(nb[v].begin(), nb[v].end());
        nb[v].erase(std::unique(nb[v].begin(), nb[v].end()), nb[v].end());
        rowPtr[v + 1] = rowPtr[v] + static_cast<int>(nb[v].size());
    }
    col.resize(rowPtr[nV]);
    diagSlot.resize(nV);
    for (int v = 0; v < nV; ++v) {
        std::copy(nb[v].begin(), nb[v].end(), col.begin() + rowPtr[v]);
        diagSlot[v] = rowPtr[v] + static_cast<int>(std::lower_bound(nb[v].begin(), nb[v].end(), v) - nb[v].begin());
        std::vector<int>().swap(nb[v]);
    }
    const int nnzb = rowPtr[nV];
    std::vector<int> slotOf(9 * (size_t)nF, -1);
    cPtr.assign(nnzb + 1, 0);
    for (int t = 0; t < nF; ++t)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int va = F[3 * t + a], vb = F[3 * t + b];
                if (fixedMask[va] || fixedMask[vb]) continue;
                const int* lo = col.data() + rowPtr[va];
                const int* hi = col.data() + rowPtr[va + 1];
                const int s = static_cast<int>(std::lower_bound(lo, hi, vb) - col.data());
                slotOf[9 * (size_t)t + 3 * a + b] = s;
                cPtr[s + 1]++;
            }
    for (int s = 0; s < nnzb; ++s) cPtr[s + 1] += cPtr[s];
    cIdx.resize(cPtr[nnzb]);
    std::vector<int> fill(cPtr.begin(), cPtr.end() - 1);
    for (int t = 0; t < nF; ++t)        // increasing t: each list in triangle order
        for (int k = 0; k < 9; ++k) {
            const int s = slotOf[9 * (size_t)t + k];
            if (s >= 0) cIdx[fill[s]++] = 9 * t + k;
        }
}

void free_bsr(oc::DeviceBsr& b)
{
    cudaFree(b.rowPtr); cudaFree(b.col); cudaFree(b.val); cudaFree(b.diagSlot); cudaFree(b.rowFixed);
    cudaFree(b.cPtr); cudaFree(b.cIdx); cudaFree(b.dinv);
    b = oc::DeviceBsr{};
}

int linsys_set_pattern(oc_linsys* ls, int nV, const int* F, int nF, const std::vector<unsigned char>& mask)
{
    oc_ctx* ctx = ls->ctx;
    std::vector<int> cPtr, cIdx;
    build_pattern(nV, F, nF, mask, ls->rowPtr, ls->col, ls->diagSlot, cPtr, cIdx);
    ls->rowFixed = mask;
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
    OC_CUDA(ctx, upload(b.rowFixed, mask.data(), nV, st));
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
        // analyze_pattern (EigenLibSolver.cpp:71-77): symbolic factorisation
        oc::chol_analyze(ls->chol, nV, ls->rowPtr.data(), ls->col.data());
        std::string err;
        int rc = oc::chol_upload(ls->chol, &err);
        if (rc) return fail(ctx, rc, err);
    }
    return OC_OK;
}

// numeric factorisation (direct) or preconditioner (PCG); fixedDiag > 0 sets
// the fixed rows' diagonal blocks to fixedDiag * I first
int linsys_factor(oc_linsys* ls, double fixedDiag, int* nBad)
{
    oc_ctx* ctx = ls->ctx;
    cudaStream_t st = ctx->stream;
    OC_CUDA(ctx, cudaMemsetAsync(ls->dFlag, 0, sizeof(int), st));
    if (fixedDiag > 0.0) oc::launch_precond_fixed(ls->b, fixedDiag, st, ls->dFlag);
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
    m->rest.resize(8 * (size_t)nF);
    // TriMesh::computeFeatures rest constants (TriMesh.cpp:343-404)
    double surfaceArea = 0.0;
    bool invalid = false;
    for (int t = 0; t < nF; ++t) {
        const double* P1 = V_rest + 3 * (size_t)F[3 * t];
        const double* P2 = V_rest + 3 * (size_t)F[3 * t + 1];
        const double* P3 = V_rest + 3 * (size_t)F[3 * t + 2];
        const double a[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]};
        const double b[3] = {P3[0] - P1[0], P3[1] - P1[1], P3[2] - P1[2]};
        const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        double* r = &m->rest[8 * (size_t)t];
        r[0] = 0.5 * std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (r[0] == 0.0) invalid = true;
        if (r[0] < areaThres) {
            r[0] = areaThres;
            surfaceArea += areaThres;
            r[1] = areaThres * areaThres;
            r[2] = r[3] = 4.0 / std::sqrt(3.0) * areaThres;
            r[4] = r[2] / 2.0;
            r[5] = r[6] = 2.0 / std::sqrt(3.0) / areaThres;
            r[7] = r[5] / 2.0;
        }
        else {
            surfaceArea += r[0];
            r[1] = r[0] * r[0];
            r[2] = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
            r[3] = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
            r[4] = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
            r[5] = r[2] / 2. / r[1];
            r[6] = r[3] / 2. / r[1];
            r[7] = r[4] / 2. / r[1];
        }
    }
    if (invalid) {
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
    // SoA upload
    oc::DeviceMesh& d = m->d;
    d.nV = nV;
    d.nF = nF;
    std::vector<int> f0(nF), f1(nF), f2(nF);
    std::vector<double> col[8];
    for (auto& c : col) c.resize(nF);
    for (int t = 0; t < nF; ++t) {
        f0[t] = F[3 * t]; f1[t] = F[3 * t + 1]; f2[t] = F[3 * t + 2];
        const double* r = &m->rest[8 * (size_t)t];
        col[0][t] = r[1];                    // triAreaSq
        col[1][t] = r[0] / surfaceArea;      // w (SymDirichletEnergy.cpp:41)
        col[2][t] = r[2]; col[3][t] = r[3]; col[4][t] = r[4];
        col[5][t] = r[5]; col[6][t] = r[6]; col[7][t] = r[7];
    }
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
    std::vector<unsigned char> mask(nV, 0);
    for (int i = 0; i < nFixed; ++i) mask[fixedVert[i]] = 1;
    cudaStream_t st = ctx->stream;
    int rc = OC_OK;
    auto chk = [&](cudaError_t e, const char* what) {
        if (rc == OC_OK && e != cudaSuccess) rc = fail(ctx, OC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    chk(dalloc(&d.F0, nF), "alloc"); chk(dalloc(&d.F1, nF), "alloc"); chk(dalloc(&d.F2, nF), "alloc");
    double** dcols[8] = {&d.A2, &d.w, &d.e0, &d.e1, &d.e01, &d.e0d, &d.e1d, &d.e01d};
    for (int k = 0; k < 8; ++k) chk(dalloc(dcols[k], nF), "alloc");
    chk(dalloc(&d.uv, nV), "alloc");
    chk(dalloc(&d.vcPtr, nV + 1), "alloc");
    chk(dalloc(&d.vcIdx, 3 * (size_t)nF), "alloc");
    chk(dalloc(&d.fixedMask, nV), "alloc");
    chk(dalloc(&m->cornerBuf, 3 * (size_t)nF), "alloc");
    chk(dalloc(&m->tmpV, nV), "alloc");
    chk(dalloc(&m->hb, 21 * (size_t)nF), "alloc");
    m->scratch.maxBlocks = 1216;
    chk(dalloc(&m->scratch.partials, (size_t)m->scratch.maxBlocks * oc::kMaxTrials), "alloc");
    chk(dalloc(&m->scratch.result, 16), "alloc");
    chk(dalloc(&m->scratch.minBits, 2), "alloc");
    chk(cudaMallocHost(&m->scratch.hostResult, sizeof(double) * 16), "alloc host");
    if (rc == OC_OK) {
        chk(upload(d.F0, f0.data(), nF, st), "upload"); chk(upload(d.F1, f1.data(), nF, st), "upload");
        chk(upload(d.F2, f2.data(), nF, st), "upload");
        for (int k = 0; k < 8; ++k) chk(upload(*dcols[k], col[k].data(), nF, st), "upload");
        chk(cudaMemcpyAsync(d.uv, UV, sizeof(double2) * nV, cudaMemcpyHostToDevice, st), "upload");
        chk(upload(d.vcPtr, vcPtr.data(), nV + 1, st), "upload");
        chk(upload(d.vcIdx, vcIdx.data(), 3 * (size_t)nF, st), "upload");
        chk(upload(d.fixedMask, mask.data(), nV, st), "upload");
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
    oc::DeviceMesh& d = m->d;
    cudaFree(d.F0); cudaFree(d.F1); cudaFree(d.F2);
    cudaFree(d.A2); cudaFree(d.w); cudaFree(d.e0); cudaFree(d.e1); cudaFree(d.e01);
    cudaFree(d.e0d); cudaFree(d.e1d); cudaFree(d.e01d);
    cudaFree(d.uv); cudaFree(d.vcPtr); cudaFree(d.vcIdx); cudaFree(d.fixedMask);
    cudaFree(m->cornerBuf); cudaFree(m->tmpV); cudaFree(m->hb); cudaFree(m->tmpF);
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
    if (!m || !blocks) return OC_ERR_INVALID;
    if (!m->tmpF) OC_CUDA(m->ctx, dalloc(&m->tmpF, 36 * (size_t)m->d.nF));
    oc::launch_hessian(m->d, uniformWeight, m->hb, m->ctx->stream);
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
    oc::chol_free(ls->chol);
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

int oc_chol_analyze_stats(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize, double* out8)
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
    oc::chol_analyze(P, nV, rowPtr.data(), col.data(), leafSize > 0 ? leafSize : 16);
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
    return OC_OK;
}

int oc_optimizer_create(oc_mesh* mesh, double energyParam, const oc_optimizer_config* cfg, oc_optimizer** out)
{
    if (!mesh || !out || !(energyParam > 0.0)) return OC_ERR_INVALID;
    oc_optimizer* o = new (std::nothrow) oc_optimizer;
    if (!o) return OC_ERR_NOMEM;
    o->mesh = mesh;
    o->param = energyParam;
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
    cudaFree(o->g); cudaFree(o->dir); cudaFree(o->uv0);
    if (o->ls) oc_linsys_destroy(o->ls);
    for (auto& e : o->ev)
        if (e) cudaEventDestroy(e);
    delete o;
    return OC_OK;
}

static void update_target_gres(oc_optimizer* o)
{
    // Optimizer::updateTargetGRes (Optimizer.cpp:675-678)
    const oc_mesh* m = o->mesh;
    o->targetGRes = o->param * static_cast<double>(m->d.nV - (int)m->fixed.size()) / static_cast<double>(m->d.nV) *
                    o->relGL2Tol;
}

static int compute_energy(oc_optimizer* o, const double2* uv, const double2* dir, const double* alphas, int n,
                          double* out)
{
    oc_mesh* m = o->mesh;
    oc::launch_energy(m->d, uv, dir, alphas, n, 0, 1.0, m->scratch, m->ctx->stream);
    o->launches += 2;
    double e[oc::kMaxTrials];
    int rc = read_result(m, n, e);
    if (rc) return rc;
    for (int k = 0; k < n; ++k) out[k] = o->param * e[k];   // Optimizer.cpp:767
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
    std::vector<unsigned char> mask(m->d.nV, 0);
    for (int v : m->fixed) mask[v] = 1;
    rc = linsys_set_pattern(o->ls, m->d.nV, m->F.data(), m->d.nF, mask);
    if (rc) return rc;
    o->lastEDec = 0.0;
    update_target_gres(o);
    rc = compute_energy(o, m->d.uv, nullptr, nullptr, 1, &o->lastEnergyVal);
    if (rc) return rc;
    o->precomputed = true;
    return OC_OK;
}

// One Newton iteration: Optimizer::solve's body (Optimizer.cpp:208-230) with
// solve_oneStep (:505-573) and lineSearch (:575-652), scaffold off.
static int solve_one(oc_optimizer* o, int* converged)
{
    oc_mesh* m = o->mesh;
    oc_ctx* ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    *converged = 0;
    record(o, 0);
    oc::launch_gradient(m->d, 0, o->param, m->cornerBuf, o->g, m->scratch, st);
    o->launches += 3;
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
    oc::launch_hessian(m->d, 0, m->hb, st);
    record(o, 2);
    oc::launch_assemble(o->ls->b, m->hb, m->d.nF, o->param, st);
    o->launches += 2;
    record(o, 3);
    // factorize (direct) or block-Jacobi preconditioner (PCG); fixed rows = param * I
    int bad = 0;
    rc = linsys_factor(o->ls, o->param, &bad);
    if (rc) return rc;
    o->badPivots = bad;
    o->launches += 1 + (o->ls->kind == OC_SOLVER_DIRECT ? 3 + (long long)o->ls->chol.launches.size() : 0);
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
    // Optimizer::lineSearch: injective bound, then halve until E <= E_last
    oc::launch_init_step(m->d, o->dir, 1.0, m->scratch, st);
    o->launches += 2;
    double step = 1.0;
    rc = read_min(m, &step);
    if (rc) return rc;
    record(o, 6);
    step *= 0.99;
    OC_CUDA(ctx, cudaMemcpyAsync(o->uv0, m->d.uv, sizeof(double2) * m->d.nV, cudaMemcpyDeviceToDevice, st));
    bool stopped = false;
    double testE = 0.0, accepted = -1.0, lastTried = step, lastTriedE = 0.0;
    int lsLaunches = 0;
    int batch = 1;
    double alpha = step;
    while (accepted < 0.0) {
        double alphas[oc::kMaxTrials], E[oc::kMaxTrials];
        int n = 0;
        for (double a = alpha; n < batch && a != 0.0; a /= 2.0) alphas[n++] = a;
        if (n == 0) break;
        rc = compute_energy(o, o->uv0, o->dir, alphas, n, E);
        if (rc) return rc;
        ++lsLaunches;
        for (int k = 0; k < n; ++k) {
            lastTried = alphas[k];
            lastTriedE = E[k];
            if (!(E[k] > o->lastEnergyVal)) {   // while(testingE > lastEnergyVal) halves, Optimizer.cpp:597
                accepted = alphas[k];
                testE = E[k];
                break;
            }
        }
        alpha = alphas[n - 1] / 2.0;
        batch = o->cfg.lineSearchBatch;
    }
    if (accepted < 0.0) {   // step reached 0 (Optimizer.cpp:600-606): keep the last trial
        stopped = true;
        accepted = lastTried;
        testE = lastTriedE;
    }
    oc::launch_step_forward(o->uv0, o->dir, accepted, m->d.uv, m->d.nV, st);
    o->launches += 1;
    OC_CUDA(ctx, cudaGetLastError());
    record(o, 7);
    o->lastEDec = o->lastEnergyVal - testE;
    if ((o->lastEDec / o->lastEnergyVal < 1.0e-6 * accepted) && (accepted > 1.0e-3)) stopped = true;   // :635-638
    o->lastEnergyVal = testE;
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
    return compute_energy(o, o->mesh->d.uv, nullptr, nullptr, 1, &o->lastEnergyVal);
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

int oc_optimizer_launch_count(oc_optimizer* o, long long* n)
{
    if (!o || !n) return OC_ERR_INVALID;
    *n = o->launches;
    return OC_OK;
}

} // extern "C"
