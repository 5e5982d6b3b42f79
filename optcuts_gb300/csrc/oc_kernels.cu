// Newton-matrix kernels of the geometry step: block-CSR assembly of the
// per-triangle Hessians (computed in oc_fp64.cu), block-Jacobi
// preconditioner, SpMV and the persistent PCG solve.
//
// Precision: FP64 throughout.  The Newton systems are extremely
// ill-conditioned (a Tutte start has UV triangles 1e-9 times their rest
// area, condition numbers near 1e14): FP32 Krylov arithmetic stalls on them,
// and an FP32-rounded matrix (or FP32 eigen-projection) moves the exact
// Newton direction by up to cond * 6e-8 in its near-null modes, which shows
// up as energy-trace differences of tens of percent against the reference.

#include "oc_internal.h"

#include <cooperative_groups.h>

#include <cmath>
#include <cstdio>

namespace cg = cooperative_groups;

namespace oc {
namespace {

// Packed symmetric 6x6: 3 diagonal 2x2 blocks (xx, xy, yy) at 0..8, then
// off-diagonal blocks (0,1), (0,2), (1,2) row-major at 9..20.
__device__ __forceinline__ int pair_index(int a, int b) { return a + b - 1; }   // (0,1)->0 (0,2)->1 (1,2)->2

// Per-triangle Hessian (SymDirichletEnergy.cpp:440-522) projected to PSD
// (IglUtils::makePD, IglUtils.hpp:71-90), all FP64.
__device__ __forceinline__ Blk2 local_block(const double* __restrict__ hb, int nF, int code)
{
    const int t = code / 9, ab = code - 9 * t, a = ab / 3, b = ab - 3 * a;
    if (a == b) {
        const double xx = hb[(3 * a) * (size_t)nF + t], xy = hb[(3 * a + 1) * (size_t)nF + t],
                     yy = hb[(3 * a + 2) * (size_t)nF + t];
        return Blk2{xx, xy, xy, yy};
    }
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const int base = 9 + 4 * pair_index(lo, hi);
    const double h00 = hb[(base + 0) * (size_t)nF + t], h01 = hb[(base + 1) * (size_t)nF + t],
                 h10 = hb[(base + 2) * (size_t)nF + t], h11 = hb[(base + 3) * (size_t)nF + t];
    return a < b ? Blk2{h00, h01, h10, h11} : Blk2{h00, h10, h01, h11};
}

__global__ void k_hessian_expand(const double* __restrict__ hb, int nF, double* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nF) return;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            const Blk2 B = local_block(hb, nF, t * 9 + a * 3 + b);
            double* o = out + 36 * (size_t)t;
            o[6 * (2 * a) + 2 * b] = B.a00;
            o[6 * (2 * a) + 2 * b + 1] = B.a01;
            o[6 * (2 * a + 1) + 2 * b] = B.a10;
            o[6 * (2 * a + 1) + 2 * b + 1] = B.a11;
        }
}

// One thread per block slot: fixed-order sum of its triangle contributions
// (the device counterpart of LinSysSolver::update_a, LinSysSolver.hpp:138-159,
// and Optimizer.cpp:825's energyParams scaling).
__global__ void __launch_bounds__(256) k_assemble(DeviceBsr b, const double* __restrict__ hb, int nF, double scale)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nnzb) return;
    Blk2 acc{0.0, 0.0, 0.0, 0.0};
    for (int p = b.cPtr[s]; p < b.cPtr[s + 1]; ++p) {
        const Blk2 B = local_block(hb, nF, b.cIdx[p]);
        acc.a00 += B.a00; acc.a01 += B.a01; acc.a10 += B.a10; acc.a11 += B.a11;
    }
    b.val[s] = Blk2{acc.a00 * scale, acc.a01 * scale, acc.a10 * scale, acc.a11 * scale};
}

// Assembly with a scaffold: the mesh's contributions (scaled by
// energyParams[0], Optimizer.cpp:825) come first in every slot list, then the
// air mesh's (scaled by w_scaf / |F_air|, Scaffold::augmentProxyMatrix,
// Scaffold.cpp:232-250, remapped to the augmented numbering).
__global__ void __launch_bounds__(256) k_assemble_scaf(DeviceBsr b, const double* __restrict__ hb, int nF, double scale,
                                                       const double* __restrict__ hbAir, int nFa, double airScale)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nnzb) return;
    Blk2 acc{0.0, 0.0, 0.0, 0.0}, accA{0.0, 0.0, 0.0, 0.0};
    for (int p = b.cPtr[s]; p < b.cPtr[s + 1]; ++p) {
        const Blk2 B = local_block(hb, nF, b.cIdx[p]);
        acc.a00 += B.a00; acc.a01 += B.a01; acc.a10 += B.a10; acc.a11 += B.a11;
    }
    for (int p = b.aPtr[s]; p < b.aPtr[s + 1]; ++p) {
        const Blk2 B = local_block(hbAir, nFa, b.aIdx[p]);
        accA.a00 += B.a00; accA.a01 += B.a01; accA.a10 += B.a10; accA.a11 += B.a11;
    }
    b.val[s] = Blk2{acc.a00 * scale + accA.a00 * airScale, acc.a01 * scale + accA.a01 * airScale,
                    acc.a10 * scale + accA.a10 * airScale, acc.a11 * scale + accA.a11 * airScale};
}

// Fixed rows: diagonal = energyParam * I (SymDirichletEnergy.cpp:541-548 scaled
// at Optimizer.cpp:825), plus w_scaf / |F_air| * I when the vertex is also a
// fixed air-mesh vertex (rowFixed == 2); block-Jacobi inverse per row.
__global__ void k_precond(DeviceBsr b, double fixedDiag, double fixedDiag2, int* flag)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b.nRows) return;
    const int s = b.diagSlot[r];
    if (b.rowFixed[r] && fixedDiag > 0.0) {
        const double d = b.rowFixed[r] == 2 ? fixedDiag2 : fixedDiag;
        b.val[s] = Blk2{d, 0.0, 0.0, d};
    }
    const Blk2 D = b.val[s];
    const double a = D.a00, bb = 0.5 * (D.a01 + D.a10), d = D.a11;
    const double det = a * d - bb * bb;
    if (a > 0.0 && det > 0.0) {
        b.dinv[r] = Mat2d{d / det, -bb / det, -bb / det, a / det};
    }
    else {
        // singular or indefinite diagonal block: fall back to a scaled identity
        const double mx = fmax(fabs(a), fabs(d));
        const double iv = mx > 0.0 ? 1.0 / mx : 1.0;
        b.dinv[r] = Mat2d{iv, 0.0, 0.0, iv};
        atomicAdd(flag, 1);
    }
}

__device__ __forceinline__ double2 row_spmv(const DeviceBsr& b, int r, const double2* __restrict__ x)
{
    double sx = 0.0, sy = 0.0;
    const int e = b.rowPtr[r + 1];
    for (int p = b.rowPtr[r]; p < e; ++p) {
        const Blk2 A = b.val[p];
        const double2 xv = x[b.col[p]];
        sx = fma(A.a00, xv.x, sx);
        sx = fma(A.a01, xv.y, sx);
        sy = fma(A.a10, xv.x, sy);
        sy = fma(A.a11, xv.y, sy);
    }
    return make_double2(sx, sy);
}

__global__ void k_spmv(DeviceBsr b, const double2* __restrict__ x, double2* __restrict__ y)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b.nRows) return;
    y[r] = row_spmv(b, r, x);
}

__device__ __forceinline__ double2 apply_dinv(const Mat2d M, const double2 v)
{
    return make_double2(M.a00 * v.x + M.a01 * v.y, M.a10 * v.x + M.a11 * v.y);
}

__device__ __forceinline__ double block_reduce_sum(double v, double* sh)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (warp == 0) {
        s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    __syncthreads();
    return s;   // valid in thread 0
}

// Persistent block-Jacobi PCG in the Chronopoulos-Gear form: one SpMV and
// one fused reduction (gamma = r.u, delta = w.u, ||r||^2) per iteration,
// two grid-wide barriers per iteration.  Every block reduces the per-block
// partials in the same fixed order, so all blocks take identical decisions
// and the result is deterministic.  The loop is capped at maxIter.
__global__ void __launch_bounds__(512) k_pcg(DeviceBsr b, const double2* __restrict__ rhs, double2* __restrict__ x,
                                             double2* __restrict__ r, double2* __restrict__ p,
                                             double2* __restrict__ z, double2* __restrict__ u,
                                             double2* __restrict__ wv, double tol2, int maxIter, double rhsSign,
                                             double* __restrict__ partials, int* status, double* outScalars)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[32];
    __shared__ double bc[4];
    const int n = b.nRows;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    for (int i = gtid; i < n; i += gstride) {
        const double2 bi = make_double2(rhsSign * rhs[i].x, rhsSign * rhs[i].y);
        x[i] = make_double2(0.0, 0.0);
        r[i] = bi;
        u[i] = apply_dinv(b.dinv[i], bi);
        p[i] = make_double2(0.0, 0.0);
        z[i] = make_double2(0.0, 0.0);
    }
    grid.sync();
    double alphaPrev = 1.0, gammaPrev = 1.0;
    double bb = -1.0, rr = 0.0;
    int it = 0;
    for (;; ++it) {
        double gam = 0.0, del = 0.0, rrl = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            const double2 wi = row_spmv(b, i, u);
            const double2 ri = r[i], ui = u[i];
            wv[i] = wi;
            gam += ri.x * ui.x + ri.y * ui.y;
            del += wi.x * ui.x + wi.y * ui.y;
            rrl += ri.x * ri.x + ri.y * ri.y;
        }
        gam = block_reduce_sum(gam, sh);
        del = block_reduce_sum(del, sh);
        rrl = block_reduce_sum(rrl, sh);
        if (threadIdx.x == 0) {
            partials[4 * blockIdx.x + 0] = gam;
            partials[4 * blockIdx.x + 1] = del;
            partials[4 * blockIdx.x + 2] = rrl;
        }
        grid.sync();
        if (threadIdx.x < 32) {
            double g3[3] = {0.0, 0.0, 0.0};
            for (int k = threadIdx.x; k < (int)gridDim.x; k += 32) {
                g3[0] += partials[4 * k + 0];
                g3[1] += partials[4 * k + 1];
                g3[2] += partials[4 * k + 2];
            }
#pragma unroll
            for (int q = 0; q < 3; ++q)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) g3[q] += __shfl_down_sync(0xffffffffu, g3[q], o);
            if (threadIdx.x == 0) { bc[0] = g3[0]; bc[1] = g3[1]; bc[2] = g3[2]; }
        }
        __syncthreads();
        gam = bc[0]; del = bc[1]; rr = bc[2];
        if (bb < 0.0) bb = rr;
        const bool done = (rr <= tol2 * bb) || !(rr == rr) || it >= maxIter;
        if (done) break;
        double beta, alpha;
        if (it == 0) { beta = 0.0; alpha = gam / del; }
        else { beta = gam / gammaPrev; alpha = gam / (del - beta * gam / alphaPrev); }
        for (int i = gtid; i < n; i += gstride) {
            const double2 ui = u[i], wi = wv[i];
            double2 pi = p[i], zi = z[i], xi = x[i], ri = r[i];
            pi.x = ui.x + beta * pi.x; pi.y = ui.y + beta * pi.y;
            zi.x = wi.x + beta * zi.x; zi.y = wi.y + beta * zi.y;
            xi.x += alpha * pi.x; xi.y += alpha * pi.y;
            ri.x -= alpha * zi.x; ri.y -= alpha * zi.y;
            p[i] = pi; z[i] = zi; x[i] = xi; r[i] = ri;
            u[i] = apply_dinv(b.dinv[i], ri);
        }
        gammaPrev = gam;
        alphaPrev = alpha;
        grid.sync();
    }
    if (gtid == 0) {
        status[0] = it;
        status[1] = (rr <= tol2 * bb) ? 1 : 0;
        outScalars[0] = rr;
        outScalars[1] = bb;
    }
}

} // namespace

void launch_hessian_expand(const double* hb, int nF, double* out, cudaStream_t st)
{
    k_hessian_expand<<<(nF + 255) / 256, 256, 0, st>>>(hb, nF, out);
}

void launch_assemble(const DeviceBsr& b, const double* hb, int nF, double scale, cudaStream_t st)
{
    k_assemble<<<(b.nnzb + 255) / 256, 256, 0, st>>>(b, hb, nF, scale);
}

void launch_assemble_scaf(const DeviceBsr& b, const double* hb, int nF, double scale, const double* hbAir, int nFa,
                          double airScale, cudaStream_t st)
{
    k_assemble_scaf<<<(b.nnzb + 255) / 256, 256, 0, st>>>(b, hb, nF, scale, hbAir, nFa, airScale);
}

int launch_precond(const DeviceBsr& b, cudaStream_t st, int* dFlag)
{
    k_precond<<<(b.nRows + 255) / 256, 256, 0, st>>>(b, -1.0, -1.0, dFlag);
    return 0;
}

void launch_precond_fixed(const DeviceBsr& b, double fixedDiag, cudaStream_t st, int* dFlag, double fixedDiag2)
{
    k_precond<<<(b.nRows + 255) / 256, 256, 0, st>>>(b, fixedDiag, fixedDiag2, dFlag);
}

void launch_spmv(const DeviceBsr& b, const double2* x, double2* y, cudaStream_t st)
{
    k_spmv<<<(b.nRows + 255) / 256, 256, 0, st>>>(b, x, y);
}

void pcg_alloc(PcgWork& wk, int nRows, int device)
{
    wk.n = nRows;
    const size_t bytes = sizeof(double2) * (size_t)(nRows > 0 ? nRows : 1);
    cudaMalloc(&wk.x, bytes);
    cudaMalloc(&wk.r, bytes);
    cudaMalloc(&wk.p, bytes);
    cudaMalloc(&wk.z, bytes);
    cudaMalloc(&wk.u, bytes);
    cudaMalloc(&wk.w, bytes);
    int nsm = 0, perSm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    wk.block = 512;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_pcg, wk.block, 0);
    if (perSm > 2) perSm = 2;
    if (perSm < 1) perSm = 1;
    wk.grid = nsm * perSm;
    const int need = (nRows + wk.block - 1) / wk.block;
    if (wk.grid > need) wk.grid = need > 0 ? need : 1;
    cudaMalloc(&wk.partials, sizeof(double) * 4 * (size_t)wk.grid + 4 * sizeof(double));
    cudaMalloc(&wk.status, sizeof(int) * 4);
}

void pcg_free(PcgWork& wk)
{
    cudaFree(wk.x); cudaFree(wk.r); cudaFree(wk.p); cudaFree(wk.z); cudaFree(wk.u); cudaFree(wk.w);
    cudaFree(wk.partials); cudaFree(wk.status);
    wk = PcgWork{};
}

int pcg_solve(const DeviceBsr& b, const double2* rhs, double2* x, PcgWork& wk, double tol, int maxIter,
              double rhsSign, cudaStream_t st, int* itersOut, double* relresOut, std::string* err)
{
    double* scal = wk.partials + 4 * (size_t)wk.grid;
    double tol2 = tol * tol;
    DeviceBsr bb = b;
    double2* xo = x;
    void* args[] = {&bb, (void*)&rhs, &xo, &wk.r, &wk.p, &wk.z, &wk.u, &wk.w, &tol2, &maxIter, &rhsSign,
                    &wk.partials, &wk.status, &scal};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_pcg, dim3(wk.grid), dim3(wk.block), args, 0, st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("PCG launch: ") + cudaGetErrorString(e);
        return OC_ERR_CUDA;
    }
    int hs[4];
    double hsc[2];
    cudaMemcpyAsync(hs, wk.status, sizeof(int) * 2, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hsc, scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("PCG: ") + cudaGetErrorString(e);
        return OC_ERR_CUDA;
    }
    if (itersOut) *itersOut = hs[0];
    if (relresOut) *relresOut = hsc[1] > 0.0 ? std::sqrt(hsc[0] / hsc[1]) : 0.0;
    return hs[1] ? 0 : OC_ERR_NOT_CONVERGED;
}

} // namespace oc
