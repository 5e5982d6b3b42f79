// Internal declarations shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include "optcuts_gpu.h"

#include <algorithm>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <atomic>
#include <pthread.h>
#include <thread>
#include <type_traits>
#include <vector>

namespace oc {

// Persistent host worker pool: up to 15 workers (16 threads with the caller)
// started on first use, so a parallel loop costs a wake-up instead of a
// thread spawn and join per worker (~0.5 ms for 15 threads).  A job is a
// count of tasks; workers and the calling thread claim tasks in index order
// under the pool's lock, the caller runs tasks until none is left and then
// waits only for tasks other threads already claimed, so a task may itself
// run a nested job (a worker caller drives its own job to completion).
// Tasks must not throw (as on a std::thread).  A forked child process gets
// a new pool (a fork handler drops the parent's, whose workers do not exist
// there).  A job of one task runs inline without touching the pool.
class HostPool {
public:
    static HostPool& get()
    {
        HostPool* p = current().load(std::memory_order_acquire);
        if (p) return *p;
        std::lock_guard<std::mutex> g(create_mu());
        p = current().load(std::memory_order_relaxed);
        if (!p) {
            static const bool hooked = [] {
                // a forked child starts without the parent's workers
                pthread_atfork(nullptr, nullptr, [] { current().store(nullptr, std::memory_order_relaxed); });
                return true;
            }();
            (void)hooked;
            p = new HostPool();   // never destroyed: its workers block forever
            current().store(p, std::memory_order_release);
        }
        return *p;
    }
    static size_t threads()
    {
        static const size_t n = std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), 16));
        return n;
    }
    void run(size_t nTasks, void (*call)(void*, size_t), void* ctx)
    {
        if (nTasks == 0) return;
        if (nTasks == 1) {
            call(ctx, 0);
            return;
        }
        start_workers();
        Job j{call, ctx, nTasks, 0, 0};
        {
            std::lock_guard<std::mutex> g(mu_);
            queue_.push_back(&j);
        }
        cv_.notify_all();
        for (;;) {
            size_t t;
            {
                std::lock_guard<std::mutex> g(mu_);
                if (j.next >= j.n) break;
                t = j.next++;
                if (j.next == j.n) queue_.erase(std::find(queue_.begin(), queue_.end(), &j));
            }
            call(ctx, t);
            finish(j);
        }
        std::unique_lock<std::mutex> lk(mu_);
        doneCv_.wait(lk, [&] { return j.done == j.n; });
    }

private:
    struct Job {
        void (*call)(void*, size_t);
        void* ctx;
        size_t n, next, done;
    };
    HostPool() = default;
    static std::atomic<HostPool*>& current()
    {
        static std::atomic<HostPool*> p{nullptr};
        return p;
    }
    static std::mutex& create_mu()
    {
        static std::mutex m;
        return m;
    }
    void start_workers()
    {
        std::lock_guard<std::mutex> g(mu_);
        if (started_) return;
        started_ = true;
        for (size_t w = 1; w < threads(); ++w) std::thread([this] { loop(); }).detach();
    }
    void finish(Job& j)
    {
        std::lock_guard<std::mutex> g(mu_);
        if (++j.done == j.n) doneCv_.notify_all();
    }
    void loop()
    {
        for (;;) {
            Job* j;
            size_t t;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return !queue_.empty(); });
                j = queue_.front();
                t = j->next++;
                if (j->next == j->n) queue_.pop_front();
            }
            j->call(j->ctx, t);
            finish(*j);
        }
    }
    bool started_ = false;
    std::mutex mu_;
    std::condition_variable cv_, doneCv_;
    std::deque<Job*> queue_;
};

// fn(t) for every t in [0, nTasks) on the host worker pool
template <class Fn>
void host_run_tasks(size_t nTasks, Fn&& fn)
{
    if (nTasks <= 1) {
        if (nTasks) fn(size_t(0));
        return;
    }
    using F = std::remove_reference_t<Fn>;
    HostPool::get().run(nTasks, [](void* c, size_t t) { (*static_cast<F*>(c))(t); },
                        const_cast<void*>(static_cast<const void*>(&fn)));
}

// fn(begin, end) over contiguous chunks of [0, n), one per host thread (up
// to 16); a single chunk below 2 * minChunk.  The chunk boundaries depend
// only on n, minChunk and the host's thread count.
template <class Fn>
void host_parallel_for(size_t n, size_t minChunk, Fn&& fn)
{
    const size_t nt = std::max<size_t>(1, std::min<size_t>(HostPool::threads(), n / std::max<size_t>(1, minChunk)));
    if (nt == 1) {
        if (n) fn(size_t(0), n);
        return;
    }
    host_run_tasks(nt, [&](size_t t) { fn(n * t / nt, n * (t + 1) / nt); });
}

// 2x2 FP64 matrix, row-major (block-Jacobi inverse of one vertex row).
struct __align__(32) Mat2d {
    double a00, a01, a10, a11;
};

// One 2x2 block of the Newton matrix, row-major.
struct __align__(32) Blk2 {
    double a00, a01, a10, a11;
};

// Line-search step sizes passed by value to the energy kernel.
struct Alphas {
    double a[8];
};

constexpr int kMaxTrials = 8;       // line-search step sizes per energy launch
constexpr int kReduceThreads = 256; // block size of the reduction kernels
// Grid cap of the block-partial reductions (152 SMs x 8 resident 256-thread
// blocks); every partials buffer holds kMaxReduceBlocks x kMaxTrials values.
constexpr int kMaxReduceBlocks = 1216;

// Device-resident triangle mesh (structure of arrays for per-triangle data,
// vertex-major double2 for UV so a corner gather is one 16-byte load).
struct DeviceMesh {
    int nV = 0, nF = 0;
    int *F0 = nullptr, *F1 = nullptr, *F2 = nullptr;   // corner vertex ids
    // FP64 rest constants in the reference's own form (TriMesh.cpp:367-393):
    // triAreaSq, the area weight triArea/surfaceArea, e0SqLen, e1SqLen,
    // e0dote1 (energy and gradient divide at use, SymDirichletEnergy.cpp:42-44)
    // and the *_div_dbAreaSq values the Hessian reads.
    double *A2 = nullptr, *w = nullptr;
    double *e0 = nullptr, *e1 = nullptr, *e01 = nullptr;
    double *e0d = nullptr, *e1d = nullptr, *e01d = nullptr;
    double* area = nullptr;                              // triArea
    double2* uv = nullptr;                              // nV
    // vertex -> incident corners (CSR, each list sorted by triangle id);
    // corner code = k * nF + t
    int *vcPtr = nullptr, *vcIdx = nullptr;
    unsigned char* fixedMask = nullptr;                 // nV
    int capV = 0, capF = 0;   // allocated vertex / triangle capacity (host bookkeeping)
};

// Reduction scratch: per-block partials then a fixed-order final pass.
struct Scratch {
    double* partials = nullptr;     // [maxBlocks * kMaxTrials]
    double* result = nullptr;       // [kMaxTrials + 8]
    double* hostResult = nullptr;   // pinned mirror
    unsigned long long* minBits = nullptr;
    int maxBlocks = 0;
};

// Full-symmetric 2x2-block CSR pattern + per-slot contribution lists.
struct DeviceBsr {
    int nRows = 0, nnzb = 0;
    int *rowPtr = nullptr, *col = nullptr;
    Blk2* val = nullptr;           // nnzb blocks (FP64)
    int* diagSlot = nullptr;       // nRows
    unsigned char* rowFixed = nullptr;
    // contributions: slot -> list of (t * 9 + a * 3 + b)
    int *cPtr = nullptr, *cIdx = nullptr;
    // scaffold air-mesh contributions, same coding over the air triangles
    // (aPtr has nnzb + 1 entries; null without a scaffold)
    int *aPtr = nullptr, *aIdx = nullptr;
    Mat2d* dinv = nullptr;         // block-Jacobi inverses (FP64)
};

// One local problem of the batched topology queries: a candidate split or
// merge evaluated on its local mesh (TriMesh::computeLocalEdDec_*).
constexpr int kLocalMaxFree = 4;    // free local vertices (8 DOF)
struct LocalProblem {
    int triOff, nTri;      // local triangles: rows of ltGlobal / ltCorner
    int vertOff, nVert;    // local vertices: rows of lvPos / lvSlot
    int initOff, nInit;    // global triangles summed for the initial energy
    int nFree, maxIter;
    double localArea;      // the local mesh's surfaceArea (local triangle order)
    double targetGRes;     // (nVert - nFixed) / nVert * 1e-6
    // bijective form: the local air loop, points [airOff, airOff + nAir) of
    // LocalBatch::apLocal / apPos (nAir 0: no air mesh); its degenerate-air
    // area clamp areaThres_AM (Scaffold.cpp:34, 150, 189)
    int airOff, nAir;
    double airThres;
};
constexpr int kLocalRaw = 16;       // raw per-problem quantities for the learned proposal
struct LocalResult {
    double eDec, initE, lastE;
    double2 pos[kLocalMaxFree];   // free vertices' final positions, by slot
    int iters, status;            // status 1: converged or stopped; 0: iteration cap; 2: non-finite
    int trials;                   // line-search energy evaluations
    // at the start and after the first Newton step: E0, ||g0||^2, first
    // step size, first-step trials, E1, max / min / mean-log / mean-log^2 of
    // the per-triangle unweighted energies e/(4w), per free slot 0 and 1:
    // |g_s|^2, g_0.g_1, triangles touching the slot, their energy
    double raw[kLocalRaw];
    long long cycles;             // SM clock cycles the problem's solve took
    int airStatus;                // bijective: loop-mesher status bits seen (0: every mesh as asked)
    int airSteiner;               // bijective: most Steiner points in one of its air meshes
};
struct LocalBatch {
    const LocalProblem* prob = nullptr;
    int nProb = 0;
    const int* ltGlobal = nullptr;     // global triangle id (rest constants)
    const int* ltCorner = nullptr;     // 3 local vertex ids per local triangle
    const double2* lvPos = nullptr;    // initial UV per local vertex
    const int* lvSlot = nullptr;       // free slot or -1 (fixed)
    const int* initTri = nullptr;
    LocalResult* out = nullptr;
    int fp32Hessian = 0;               // project element Hessians in FP32
    // bijective form: per air-loop point, the local vertex it is (>= 0) or
    // -1 for a fixed air point at apPos
    const int* apLocal = nullptr;
    const double2* apPos = nullptr;
};

struct PcgWork {
    double2 *x = nullptr, *r = nullptr, *p = nullptr, *z = nullptr, *u = nullptr, *w = nullptr;
    double* partials = nullptr;    // [grid * 4]
    int* status = nullptr;         // [4] iterations, flag
    int grid = 0, block = 0, n = 0;
};

// the stream of a context (oc_api.cu)
cudaStream_t ctx_stream(oc_ctx* ctx);

// ---- launchers (kernels live in oc_fp64.cu / oc_kernels.cu) ----
// energy at uv + alpha_k * dir for k < nTrials (dir may be null: alphas ignored)
// (sums go to s.result, or to out when given)
void launch_energy(const DeviceMesh& m, const double2* uv, const double2* dir, const double* alphasHost,
                   int nTrials, int uniform, double scale, Scratch& s, cudaStream_t st, double* out = nullptr);
void launch_energy_elem(const DeviceMesh& m, int uniform, double* out, cudaStream_t st);
// corner gradients (3 x nF double2) then per-vertex gather; writes ||g||^2 to s.result[0]
void launch_gradient(const DeviceMesh& m, int uniform, double scale, double2* cornerBuf, double2* g,
                     Scratch& s, cudaStream_t st);
// augmented gradient with a scaffold (Optimizer.cpp:783-797): mesh corners
// times scale, plus the air mesh's (uniform weights) times airScale on the
// boundary and air-only vertices; g and ||g||^2 over air.nV vertices
void launch_gradient_scaf(const DeviceMesh& m, double scale, double2* cornerBuf, const DeviceMesh& air,
                          double airScale, double2* airCornerBuf, double2* g, Scratch& s, cudaStream_t st);
// min over triangles of the inversion-free bound, starting from stepSize;
// with reset = false the running minimum of an earlier launch is lowered
void launch_init_step(const DeviceMesh& m, const double2* dir, double stepSize, Scratch& s, cudaStream_t st,
                      bool reset = true);
void launch_step_forward(const double2* uv0, const double2* dir, double alpha, double2* uv, int nV,
                         cudaStream_t st);
void launch_check_inversion(const DeviceMesh& m, Scratch& s, cudaStream_t st);
void launch_reduce_final(Scratch& s, int nBlocks, int nVals, cudaStream_t st, double* out = nullptr);
int reduce_blocks_for(int n);

// batched projected-Newton solves of the topology candidates' local
// problems: tpp threads per problem, or per block of a cluster of `cluster`
// blocks (schedules 8/1, 32/1, 128/1, 64/2..16);
// local_schedule picks one for a size class (largest triangle count, number
// of problems), local_max_cluster is 16 where the device runs 16-block
// clusters of this kernel, else 8
struct LocalSchedule {
    int tpp = 32, cluster = 1, block = 128;   // block: threads per block (several problems for tpp <= 32)
};
LocalSchedule local_schedule(int maxTri, int count, int numSMs, int maxCluster);
int local_max_cluster();
cudaError_t launch_local_newton(const DeviceMesh& m, double surfaceArea, const LocalBatch& b, LocalSchedule sc,
                                cudaStream_t st);
// the bijective form (problems with an air loop): one warp per problem, the
// loop re-meshed at the start of every local Newton iteration
cudaError_t launch_local_newton_bij(const DeviceMesh& m, double surfaceArea, const LocalBatch& b, cudaStream_t st);
// SymDirichletEnergy::computeDivGradPerVert (standard-deviation filter) into divGrad (nV)
void launch_divgrad(const DeviceMesh& m, double2* cornerBuf, double* divGrad, cudaStream_t st);

// per-triangle PSD-projected Hessian: 21 FP64 values per triangle (SoA)
// element Hessians with the PSD projection: OC_HESSIAN_JACOBI6 the 6x6
// cyclic Jacobi without FMA contraction (oc_fp64.cu), OC_HESSIAN_REDUCED the
// translation-free 4x4 form, OC_HESSIAN_HYBRID the 4x4 form where the
// element's energy density is at most kHybridDensity and the 6x6 form
// elsewhere (both oc_local.cu)
void launch_hessian(const DeviceMesh& m, int uniform, double* hb, cudaStream_t st,
                    int projection = OC_HESSIAN_JACOBI6);
// density <= 0: the 4x4 form everywhere
void launch_hessian_reduced(const DeviceMesh& m, int uniform, double* hb, cudaStream_t st, double density);
// symmetric Dirichlet energy density (4 at an isometry) above which the
// hybrid projection keeps the 6x6 form
constexpr double kHybridDensity = 1e3;
// expand the 21 packed values to full 6x6 FP64 (for the API / tests)
void launch_hessian_expand(const double* hb, int nF, double* out, cudaStream_t st);
void launch_assemble(const DeviceBsr& b, const double* hb, int nF, double scale, cudaStream_t st);
// mesh contributions (cPtr/cIdx) from hb times scale plus the air mesh's
// (aPtr/aIdx) from hbAir times airScale
void launch_assemble_scaf(const DeviceBsr& b, const double* hb, int nF, double scale, const double* hbAir, int nFa,
                          double airScale, cudaStream_t st);
int launch_precond(const DeviceBsr& b, cudaStream_t st, int* dFlag);
// fixed rows get fixedDiag * I (rowFixed == 1) or fixedDiag2 * I (rowFixed == 2)
void launch_precond_fixed(const DeviceBsr& b, double fixedDiag, cudaStream_t st, int* dFlag,
                          double fixedDiag2 = 0.0);
// solves A x = rhsSign * rhs (rhsSign = -1 gives the Newton direction from g)
int pcg_solve(const DeviceBsr& b, const double2* rhs, double2* x, PcgWork& wk, double tol, int maxIter,
              double rhsSign, cudaStream_t st, int* itersOut, double* relresOut, std::string* err);
void pcg_alloc(PcgWork& wk, int nRows, int device);
void pcg_free(PcgWork& wk);
void launch_spmv(const DeviceBsr& b, const double2* x, double2* y, cudaStream_t st);

} // namespace oc
