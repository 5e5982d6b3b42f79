/* optcuts_gpu.h -- C ABI of the GB300 (sm_103a) OptCuts geometry step.
 *
 * One GPU, one process.  Every entry point takes plain pointers and sizes,
 * returns an int status (oc_status), and never throws.  Host pointers are
 * caller-owned; device state lives behind opaque handles.
 *
 * Layouts follow the reference's own conventions:
 *   V_rest   nV x 3 row-major float64  (TriMesh::V_rest, src/TriMesh.hpp:30)
 *   UV       nV x 2 row-major float64  (TriMesh::V, src/TriMesh.hpp:31)
 *   F        nF x 3 row-major int32    (TriMesh::F, src/TriMesh.hpp:32)
 *   gradient / search direction: 2*nV interleaved [u0, v0, u1, v1, ...]
 *            (src/Energy/SymDirichletEnergy.cpp:262, src/Optimizer.cpp:666-669)
 *   fixed vertices: list of vertex ids (TriMesh::fixedVert, src/TriMesh.hpp:56)
 *
 * Precision: the geometry step is float64 throughout -- energies,
 * gradients, the per-triangle 6x6 Hessians and their PSD projection, the
 * assembled Newton matrix, its LDL^T factorization and substitutions, the
 * injective-step roots and the line search.  The local topology solves are
 * float64 with an optional float32 element-Hessian projection
 * (OC_TOPO_FP32_HESSIAN); the learned proposal's network computes in bf16
 * with float32 accumulation.
 */
#ifndef OPTCUTS_GPU_H
#define OPTCUTS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    OC_OK = 0,
    OC_ERR_INVALID = 1,          /* bad argument / size / index */
    OC_ERR_INVERTED = 2,         /* inverted UV triangle (Optimizer.cpp:65-67 exits) */
    OC_ERR_NOT_CONVERGED = 3,    /* PCG hit its iteration cap */
    OC_ERR_TIMEOUT = 4,          /* a device loop hit its clock budget */
    OC_ERR_BOUNDS = 5,           /* index out of range (checked builds) */
    OC_ERR_CUDA = 6,             /* CUDA runtime error; see oc_last_error() */
    OC_ERR_DEGENERATE = 7,       /* zero-area rest triangle (TriMesh.cpp:399-402 exits) */
    OC_ERR_NOT_SPD = 8,          /* non-positive diagonal block in the Newton matrix */
    OC_ERR_NOMEM = 9
} oc_status;

typedef struct oc_ctx oc_ctx;
typedef struct oc_mesh oc_mesh;
typedef struct oc_linsys oc_linsys;
typedef struct oc_optimizer oc_optimizer;

/* ---- context ---------------------------------------------------------- */
/* stream: a cudaStream_t, or NULL for a stream owned by the context. */
int oc_ctx_create(int device, void* stream, oc_ctx** out);
int oc_ctx_destroy(oc_ctx* ctx);
const char* oc_last_error(const oc_ctx* ctx);
const char* oc_status_string(int status);
int oc_ctx_synchronize(oc_ctx* ctx);

/* ---- mesh: TriMesh state on the device ---------------------------------
 * Replaces the TriMesh data the hot path reads (TriMesh.hpp:30-63) and
 * TriMesh::computeFeatures' rest constants (TriMesh.cpp:343-404).
 * areaThres: TriMesh::areaThres_AM (0 for surface meshes). */
int oc_mesh_create(oc_ctx* ctx, const double* V_rest, const double* UV, int nV,
                   const int* F, int nF, const int* fixedVert, int nFixed,
                   double areaThres, oc_mesh** out);
int oc_mesh_destroy(oc_mesh* mesh);
int oc_mesh_set_uv(oc_mesh* mesh, const double* UV);        /* host -> device */
int oc_mesh_get_uv(oc_mesh* mesh, double* UV);              /* device -> host */
/* rest: nF x 8 (triArea, triAreaSq, e0SqLen, e1SqLen, e0dote1, e0SqLen_div_dbAreaSq,
 * e1SqLen_div_dbAreaSq, e0dote1_div_dbAreaSq); scalars: surfaceArea, avgEdgeLen,
 * virtualRadius (TriMesh.cpp:343-404). Either pointer may be NULL. */
int oc_mesh_rest_constants(oc_mesh* mesh, double* rest, double* scalars);
/* TriMesh::checkInversion (TriMesh.cpp:1710-1756): *ok = 1 if every UV triangle
 * has signed double area >= 0. */
int oc_mesh_check_inversion(oc_mesh* mesh, int* ok);

/* ---- Energy: SymDirichletEnergy (Energy.hpp:27-44) -------------------- */
/* Energy::computeEnergyVal (Energy.cpp:35-40) */
int oc_sd_energy(oc_mesh* mesh, int uniformWeight, double* energyVal);
/* SymDirichletEnergy::getEnergyValPerElem (SymDirichletEnergy.cpp:24-46) */
int oc_sd_energy_per_elem(oc_mesh* mesh, int uniformWeight, double* energyValPerElem);
/* SymDirichletEnergy::computeGradient (SymDirichletEnergy.cpp:258-304); 2*nV */
int oc_sd_gradient(oc_mesh* mesh, int uniformWeight, double* gradient);
/* SymDirichletEnergy::computeHessian (SymDirichletEnergy.cpp:429-549) per
 * triangle, PSD-projected (IglUtils::makePD, IglUtils.hpp:71-90): out nF x 36
 * row-major 6x6 in local order (u1,v1,u2,v2,u3,v3), before fixed-vertex
 * removal and before energyParams scaling. */
int oc_sd_hessian_blocks(oc_mesh* mesh, int uniformWeight, double* blocks);
/* The PSD projection of the element Hessians:
 *   OC_HESSIAN_REDUCED  H = Q K Q^T with K = Q^T H Q over the 4-dimensional
 *                       complement of the two translations (Q orthonormal),
 *                       K clamped by a 4x4 cyclic Jacobi: the same projection
 *                       as the 6x6 eigen-clamp up to rounding (about 1e-15 of
 *                       each block's largest entry), at a fifth of its FP64
 *                       arithmetic
 *   OC_HESSIAN_JACOBI6  the 6x6 cyclic Jacobi eigen-clamp without FMA
 *                       contraction (rounds as the oracle restatement does);
 *                       the optimizer's default and oc_sd_hessian_blocks's
 *                       form
 *   OC_HESSIAN_HYBRID   the 4x4 form for elements whose energy density is at
 *                       most 1e3, the 6x6 form for the rest
 * The 6x6 form keeps each element's rounding-level translation components;
 * for the stiff elements of a Tutte start (entries up to ~1e26) they change
 * the Newton direction, and Newton runs with the 4x4 form everywhere
 * converge far more slowly from such starts.  Where no element is stiff the
 * three forms agree to rounding. */
enum { OC_HESSIAN_REDUCED = 0, OC_HESSIAN_JACOBI6 = 1, OC_HESSIAN_HYBRID = 2 };
enum { OC_ORDER_AUTO = 0, OC_ORDER_BFS = 1 };
/* oc_sd_hessian_blocks with the projection chosen */
int oc_sd_hessian_blocks_projected(oc_mesh* mesh, int uniformWeight, int projection, double* blocks);
/* SymDirichletEnergy::initStepSize (SymDirichletEnergy.cpp:551-610): lowers
 * *stepSize in place to the largest inversion-free step along searchDir. */
int oc_sd_init_step_size(oc_mesh* mesh, const double* searchDir, double* stepSize);

/* Allocation-free energy evaluation.  It has no counterpart in the
 * reference: it is an addition for callers that cannot allocate device
 * memory themselves -- e.g. code running inside a host framework that owns
 * every allocation, or work recorded into an externally managed CUDA graph.
 * Computes, on the given stream, E_k = sum over triangles of the symmetric
 * Dirichlet energy at UV + alphas[k] * dir for k < nTrials (dir NULL: the
 * energy at UV).  All pointers except `alphas` (host, nTrials values) are DEVICE pointers
 * owned by the caller:
 *   F        nF x 3 int32 row-major       UV, dir   nV x 2 float64 row-major
 *   rest     nF x 8 float64, the layout of oc_mesh_rest_constants
 *   energies nTrials float64 (output; unweighted by energyParams)
 * surfaceArea is TriMesh::surfaceArea (the area weights' normaliser).
 * It calls no cudaMalloc/cudaFree: block partial sums go to a static device
 * array sized for 1216 blocks x 8 trials (76 KB, held by every GPU that loads
 * the library until exit).  nTrials must be 1..8 (else OC_ERR_INVALID).
 * The first call on each device looks the array's address up
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Every call shares the array: calls that overlap on the GPU (different
 * streams, no ordering) race and must be serialised by the caller. */
int oc_sd_energy_trials_noalloc(const int* F, const double* UV, const double* dir, const double* rest,
                                double surfaceArea, int nF, const double* alphas, int nTrials, int uniformWeight,
                                double* energies, void* stream);

/* ---- LinSysSolver (LinSysSolver.hpp:22-187, EigenLibSolver.cpp:21-107) --
 * Full-symmetric 2x2-block CSR on the device.  Two solvers:
 *   OC_SOLVER_DIRECT  multifrontal sparse Cholesky (FP64 fronts), the exact
 *                     solve SimplicialLDLT performs in the reference (default)
 *   OC_SOLVER_PCG     block-Jacobi preconditioned conjugate gradients */
enum { OC_SOLVER_DIRECT = 0, OC_SOLVER_PCG = 1 };
int oc_linsys_create(oc_ctx* ctx, oc_linsys** out);
int oc_linsys_destroy(oc_linsys* ls);
/* set_type(threadAmt, mtype) (LinSysSolver.hpp:35): selects the solver;
 * call before set_pattern. */
int oc_linsys_set_type(oc_linsys* ls, int solverKind);
/* analyze_pattern() (EigenLibSolver.cpp:71-77): symbolic factorisation
 * (nested dissection, front structure); set_pattern runs it implicitly. */
int oc_linsys_analyze_pattern(oc_linsys* ls);
/* No reference counterpart (a launch choice of the direct solver): the
 * largest thread-block cluster (1..8 CTAs) per front that the substitutions
 * of the top tree levels use; 1 keeps one CTA per front everywhere.  The
 * solution is the same bits for every value.  Default 8. */
int oc_linsys_set_solve_cluster(oc_linsys* ls, int maxCluster);
/* Tree levels of the current plan whose substitutions run as clusters, and
 * the largest cluster size among them (1 when none). */
int oc_linsys_solve_clusters(oc_linsys* ls, int* levels, int* largest);
/* No reference counterpart (a launch choice of the direct solver): the most
 * CUDA streams (1..8) the factorization's independent subtrees may run on,
 * from the next analysis (set_pattern) on.  The factor is the same bits for
 * every value.  Default 8. */
int oc_linsys_set_factor_streams(oc_linsys* ls, int streams);
/* Streams and subtree groups the current plan's factorization uses. */
int oc_linsys_factor_streams(oc_linsys* ls, int* streams, int* groups);
/* Symbolic statistics of the direct solver: out[0..7] = fronts, tree levels,
 * largest front rows, front pool doubles, factor flops, tiled launches,
 * factor entries (sum of m*k), DOF. */
int oc_linsys_stats(oc_linsys* ls, double* out8);
/* The same symbolic analysis without any device call (host only). */
int oc_chol_analyze_stats(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize,
                          double* out8);
/* the same with the geometric nested dissection: vertex coordinates xy
 * (nV x 2) bisected at the median along the longer extent (the ordering the
 * optimizer uses for a scaffold's full pattern) */
int oc_chol_analyze_stats_xy(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize,
                             const double* xy, double* out8);
/* No reference counterpart (a check of the direct solver's launch plan),
 * host only: the same analysis with at most maxStreams (1..8) factorization
 * streams; out3 = streams used, subtree groups, and 1 when every front's
 * children finish before it under the plan's streams and event waits. */
int oc_chol_analyze_groups(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize,
                           int maxStreams, int* out3);
/* Its vertex elimination order (nV entries), host only. */
int oc_chol_analyze_order(int nV, const int* F, int nF, const int* fixedVert, int nFixed, int leafSize,
                          int* vertexOrder);
/* set_pattern(vNeighbor, fixedVert) (LinSysSolver.hpp:37-135): the vertex
 * adjacency is taken from the triangles F; fixed rows keep only the diagonal. */
int oc_linsys_set_pattern(oc_linsys* ls, int nV, const int* F, int nF,
                          const int* fixedVert, int nFixed);
/* update_a(I, J, V) (LinSysSolver.hpp:138-159): triplets with I <= J are summed
 * into the matrix (mirrored to the lower half), the rest are ignored. */
int oc_linsys_update_a(oc_linsys* ls, const int* I, const int* J, const double* V, int nTriplets);
/* LinSysSolver::set_pattern(vNeighbor, fixedVert) (LinSysSolver.hpp:37-135,
 * called by Optimizer.cpp:174, 358, 524): the pattern from per-vertex
 * neighbour lists (CSR: the neighbours of v are nbIdx[nbPtr[v] .. nbPtr[v+1]),
 * either or both directions of a pair may be listed); fixed vertices keep
 * only their diagonal block.  Then analyze_pattern as oc_linsys_set_pattern. */
int oc_linsys_set_pattern_neighbors(oc_linsys* ls, int nV, const int* nbPtr, const int* nbIdx, const int* fixedVert,
                                   int nFixed);
/* factorize() (EigenLibSolver.cpp:80-93): numeric Cholesky (direct) or the
 * block-Jacobi preconditioner (PCG).  OC_ERR_NOT_SPD if a pivot or diagonal
 * block was not positive (the factorisation still completes). */
int oc_linsys_factorize(oc_linsys* ls);
/* solve(rhs, result) (EigenLibSolver.cpp:96-107).  Direct: tol / maxIter are
 * ignored, *iters = 0 and *relres = the computed relative residual.  PCG: to
 * relative residual tol (<= 0: 1e-8) within maxIter (<= 0: 20000).  iters /
 * relres may be NULL. */
int oc_linsys_solve(oc_linsys* ls, const double* rhs, double* result, double tol, int maxIter,
                    int* iters, double* relres);
/* multiply(x, Ax) (LinSysSolver.hpp:172-187) */
int oc_linsys_multiply(oc_linsys* ls, const double* x, double* Ax);

/* ---- Optimizer (Optimizer.hpp:74-142) -----------------------------------
 * energyParam = energyParams[0] = 1 - lambda.  The mesh is borrowed (its UV
 * is the optimizer's `result.V`).  With a scaffold set (see
 * oc_optimizer_set_scaffold) the optimizer runs the reference's
 * scaffolding branches; w_scaf = 0.01 * energyParam at creation
 * (Optimizer.cpp:87). */
typedef struct {
    double pcgTol;        /* relative residual, default 1e-8 */
    int pcgMaxIter;       /* default 20000 */
    double relGL2Tol;     /* Optimizer.cpp:70, default 1e-12 */
    int lineSearchBatch;  /* trial step sizes per energy launch, 1..8, default 4 */
    int timing;           /* 1: record per-phase CUDA-event times */
    int linearSolver;     /* OC_SOLVER_DIRECT (default) or OC_SOLVER_PCG */
    int scaffoldPattern;  /* 0 (default): a small scaffold's boundary and air
                             vertices form one dense block, so rebuilding the
                             air mesh keeps the analysis; 1: always the exact
                             pattern (analysed again when the air mesh's
                             connectivity changes) */
    int hessianProjection; /* OC_HESSIAN_JACOBI6 (default), OC_HESSIAN_REDUCED or
                              OC_HESSIAN_HYBRID */
    int ordering;         /* direct solver's nested dissection: OC_ORDER_AUTO
                             (default: at every node the smaller balanced
                             separator of a BFS level set and a bisection of
                             the current UV positions) or OC_ORDER_BFS */
    int carryAnalysis;    /* 1 (default): after a topology operation the direct
                             solver's dissection tree is carried over (a copy
                             joins its source vertex's node, a merged vertex
                             the nodes' common ancestor) and only the front
                             structures are rebuilt; a full analysis when the
                             tree no longer separates the pattern, after 64
                             carried analyses or once the factor cost grew 30%.
                             A scaffold past the dense-clique size then keeps
                             its air-only vertices in the root front (its air
                             meshes' patterns change the front structures
                             only); 0: a full analysis after every operation
                             and every new air pattern */
} oc_optimizer_config;

int oc_optimizer_default_config(oc_optimizer_config* cfg);
int oc_optimizer_create(oc_mesh* mesh, double energyParam, const oc_optimizer_config* cfg,
                        oc_optimizer** out);
int oc_optimizer_destroy(oc_optimizer* opt);
/* Optimizer::precompute (Optimizer.cpp:154-201) */
int oc_optimizer_precompute(oc_optimizer* opt);
/* Optimizer::solve (Optimizer.cpp:203-261): *result = 0 (not converged) or
 * 1 (converged, or the line search stopped).  A zero or non-finite pivot in
 * the Newton matrix's factorization ends the call with OC_ERR_NOT_SPD
 * before any step is taken (the reference dumps the matrix and exits,
 * Optimizer.cpp:548-554); oc_optimizer_bad_pivots reports the count. */
int oc_optimizer_solve(oc_optimizer* opt, int maxIter, int* result);
/* Pivots of the last factorization that were zero or non-finite (replaced
 * by 1e-300 inside the factorization so that it completes). */
int oc_optimizer_bad_pivots(oc_optimizer* opt, int* nBad);
/* Optimizer::getLastEnergyVal (Optimizer.cpp:845-850) */
int oc_optimizer_get_last_energy(oc_optimizer* opt, double* energy);
int oc_optimizer_get_iter_num(oc_optimizer* opt, int* iterNum);
/* Optimizer::setRelGL2Tol (Optimizer.cpp:142-147) */
int oc_optimizer_set_rel_gl2_tol(oc_optimizer* opt, double tol);
/* energyParams[0] changed by the caller, then updateEnergyData(true, false,
 * false) (Optimizer.cpp:323-334; main.cpp:764). */
int oc_optimizer_set_energy_param(oc_optimizer* opt, double energyParam);
/* Last iteration's diagnostics: accepted step, PCG iterations (0 for the
 * direct solver) and relative residual, line-search energy launches, ||g||^2
 * at its start. */
int oc_optimizer_last_step(oc_optimizer* opt, double* stepSize, int* pcgIters, double* pcgRelRes,
                           int* lineSearchLaunches, double* gradSqNorm);
/* Per-phase device milliseconds accumulated since the last call (timing=1):
 * out[0..6] = gradient, hessian+projection (matrixComputation), block
 * assembly (matrixAssembly), numeric factorisation or PCG preconditioner
 * (numericalFactorization), solve (backSolve), injective step, line search
 * (lineSearch) -- the reference's timer_step buckets, main.cpp:1557-1565. */
int oc_optimizer_phase_ms(oc_optimizer* opt, double* out7);
/* Kernel launches this optimizer issued since creation (for accounting). */
int oc_optimizer_launch_count(oc_optimizer* opt, long long* launches);
/* oc_linsys_stats of the optimizer's own solver (after precompute). */
int oc_optimizer_solver_stats(oc_optimizer* opt, double* out8);
/* oc_linsys_set_solve_cluster on the optimizer's own solver. */
int oc_optimizer_set_solve_cluster(oc_optimizer* opt, int maxCluster);
/* oc_linsys_solve_clusters on the optimizer's own solver. */
int oc_optimizer_solve_clusters(oc_optimizer* opt, int* levels, int* largest);
/* oc_linsys_set_factor_streams on the optimizer's own solver (call before
 * precompute to cover every analysis). */
int oc_optimizer_set_factor_streams(oc_optimizer* opt, int streams);
/* oc_linsys_factor_streams on the optimizer's own solver. */
int oc_optimizer_factor_streams(oc_optimizer* opt, int* streams, int* groups);

/* ---- Scaffold (Scaffold.hpp:18-70; Optimizer.cpp scaffolding branches) ---
 * Replaces `scaffold = Scaffold(result, UV_bnds, E, bnd)` (Optimizer.cpp:
 * 157-161, 251-257): the caller passes the air mesh Scaffold's constructor
 * builds (Scaffold.cpp:27-205), i.e. airMesh.V (nAirV x 2, row-major), airMesh.F
 * (nAirF x 3) and bnd (air vertex i < nBnd is mesh vertex bnd[i]; rows
 * 0..nBnd-1 of airV are those vertices' current UV, as Triangle returns its
 * input points first).  Air-only vertex i >= nBnd becomes system vertex
 * nV + i - nBnd (localVI2Global).  areaThres < 0 selects the whole-mesh
 * areaThres_AM = sqrt(3)/4 (avgEdgeLen/2)^2 (Scaffold.cpp:34, 189).  The
 * mesh's fixed vertices on the boundary are fixed in the air mesh too.
 * The next solve() then includes w_scaf/|F_air| * E_SD(air mesh, uniform
 * weights) in energy, gradient, Hessian, injective step and line search.
 * The reference rebuilds the scaffold after every iteration; a caller that
 * does not call this again keeps the air mesh as the last step moved it.
 * The Newton-matrix pattern and its analysis are rebuilt on the next solve
 * when the air connectivity differs from the previous call's. */
int oc_optimizer_set_scaffold(oc_optimizer* opt, const double* airV, int nAirV, const int* airF, int nAirF,
                              const int* bnd, int nBnd, double areaThres);
/* `scaffold = Scaffold(result)` done here: the air mesh of the mesh's
 * current UV from the project's own generator (oc_air_mesh_build, 20 degree
 * refinement), then oc_optimizer_set_scaffold with the whole-mesh
 * areaThres_AM. */
int oc_optimizer_rebuild_scaffold(oc_optimizer* opt);
/* Optimizer::setScaffolding(false) (Optimizer.cpp:307-317) */
int oc_optimizer_clear_scaffold(oc_optimizer* opt);
/* The current scaffold (Optimizer::getScaffold, Optimizer.cpp:118-124):
 * sizes, and into non-NULL arrays airMesh.V as the last step moved it
 * (nAirV x 2), airMesh.F (nAirF x 3) and bnd (nBnd).  OC_ERR_INVALID
 * without a scaffold. */
int oc_optimizer_get_scaffold(oc_optimizer* opt, int* nAirV, int* nAirF, int* nBnd, double* airV, int* airF,
                              int* bnd);
/* energyVal_scaffold of the last evaluation; getLastEnergyVal(true) is
 * oc_optimizer_get_last_energy minus this (Optimizer.cpp:845-850) */
int oc_optimizer_get_last_energy_scaffold(oc_optimizer* opt, double* scaffoldEnergy);
/* vertices of the Newton system (wholeMeshSize with a scaffold, else nV) */
int oc_optimizer_system_size(oc_optimizer* opt, int* nVerts);
/* gradient and searchDir of the last iteration (2 x system size each,
 * interleaved u, v; either may be NULL) */
int oc_optimizer_last_vectors(oc_optimizer* opt, double* gradient, double* searchDir);

/* ---- Topology queries (TriMesh::querySplit / queryMerge, TriMesh.cpp:548-951)
 * The candidates of one outer-loop topology step, each scored by its exact
 * local projected-Newton solve (TriMesh::computeLocalLDec and
 * computeLocalEdDec_inSplit / _bSplit / _merge, TriMesh.cpp:2105-2862),
 * all local solves in one batched device launch.  This is the
 * bijectivity-off form (no local air meshes).  opType: */
enum { OC_OP_BOUNDARY_SPLIT = 0, OC_OP_INTERIOR_SPLIT = 1, OC_OP_MERGE = 2 };
typedef struct oc_topo_result oc_topo_result;
/* TriMesh::cohE (nCohE x 4), needed by merge queries */
int oc_mesh_set_cohesive_edges(oc_mesh* mesh, const int* cohE, int nCohE);
/* The first topology query after a change of the mesh's triangles builds
 * their vertex adjacency, the later ones reuse it; this drops it, so the
 * next query pays for it again (timing a topology step as it follows an
 * applied operation). */
int oc_mesh_drop_adjacency(oc_mesh* mesh);
/* SymDirichletEnergy::computeDivGradPerVert (SymDirichletEnergy.cpp:108-147)
 * at the mesh's current UV: the split filter, nV values */
int oc_mesh_split_filter(oc_mesh* mesh, double* divGrad);
/* querySplit(lambda_t, false, opType == OC_OP_INTERIOR_SPLIT) or
 * queryMerge(lambda_t).  lambda_t as the reference passes it
 * (1 - energyParams[0]); filterExp = filterExp_in (<= 0: 0.6).
 * options: OC_TOPO_FP32_HESSIAN projects the local element Hessians in
 * FP32 (about 8x faster local solves; energies, gradients, line search and
 * the local LDL^T stay FP64; energy changes then agree with the FP64
 * evaluation to ~1e-4 relative instead of ~1e-8). */
enum { OC_TOPO_FP32_HESSIAN = 1, OC_TOPO_RECORD_FEATURES = 2, OC_TOPO_AUTOTUNE = 8, OC_TOPO_BIJECTIVE = 16 };
/* OC_TOPO_BIJECTIVE: the bijective form, as the reference queries when its
 * TriMesh has a scaffold (bijectivity on; TriMesh.cpp:2322-2372,
 * 2406-2497, 2597-2756): each candidate's split copies are first moved
 * apart along their inward normals, and its local solve carries an air
 * mesh of the candidate's air loop -- the slit an interior split opens,
 * the split vertex's air fan opened at a boundary split
 * (Scaffold::get1RingAirLoop), the corner loop of a merge
 * (Scaffold::getCornerAirLoop, merges that close a diamond excepted) --
 * re-meshed from the current layout at every local Newton iteration (the
 * mesher of oc_air_loop_mesh), weighted 0.01 / |F_air| with uniform
 * weights.  Problems the reference abandons (air loops that share a vertex
 * or self-intersect) report an energy decrease of -DBL_MAX.  The air loops
 * come from the scaffold of the Optimizer last given this mesh
 * (oc_optimizer_set_scaffold / _rebuild_scaffold); OC_ERR_INVALID without
 * one.  With the learned proposal, the probe is the bijective solve's own
 * first iteration (features of the local mesh alone, as without air
 * loops); a network for bijective queries is trained on pairs that
 * bijective queries recorded. */
int oc_topology_query(oc_mesh* mesh, int opType, double lambda_t, double filterExp, int options, oc_topo_result** out);
/* No counterpart in the reference: the learned proposal.  Every local
 * problem first gets one Newton step (its features: energies, gradient
 * split between the split copies, first-step decrease, ...; 32 values),
 * the MLP predicts the fraction of its excess energy the full solve would
 * remove, the predicted E_w decreases are ranked and only the top fraction
 * topFrac of the problems is solved exactly (at least 32 of them, or all of
 * an operation that has fewer); the exact solves alone decide the
 * candidates' values (unsolved candidates report -DBL_MAX). */
typedef struct oc_mlp oc_mlp;
int oc_topology_query_learned(oc_mesh* mesh, int opType, double lambda_t, double filterExp, int options, oc_mlp* mlp,
                              double topFrac, oc_topo_result** out);
/* One topology step's three queries on the same state — boundary split,
 * merge, interior split (querySplit / queryMerge / querySplit(splitInterior),
 * as createFracture with and without allowInSplit ask for them) — built
 * together and solved in the same launches; each result equals its own
 * query's.  mlp NULL: exhaustive (options as oc_topology_query); else the
 * learned proposal with the top fraction topFrac of each operation's local
 * problems solved exactly. */
int oc_topology_step(oc_mesh* mesh, double lambda_t, double filterExp, int options, oc_mlp* mlp, double topFrac,
                     oc_topo_result** split, oc_topo_result** merge, oc_topo_result** interior);
/* per local problem (rows): the 32 features, the exact target (fraction of
 * the local excess energy removed; queries with OC_TOPO_RECORD_FEATURES)
 * and the MLP's prediction (learned queries); NULL arrays are skipped */
int oc_topo_result_features(const oc_topo_result* r, int* nRows, float* X, float* target, float* predicted);
/* learned queries: problems solved exactly, ms of the one-step pass and of
 * the exact solves */
int oc_topo_result_timing(const oc_topo_result* r, int* nSelected, double* probeMs, double* exactMs);
/* host phases of the query's step (ms, shared by the operations queried
 * together): out4 = inputs (positions, split filter, adjacency, air-mesh
 * copies), air-loop sources, ranking (features, MLP, selection; learned
 * queries), candidate lists */
int oc_topo_result_host_phases(const oc_topo_result* r, double* out4);
/* per local problem: its candidate, its exact E_w decrease (NaN where the
 * learned proposal did not solve it) and the predicted decrease (learned
 * queries; else NaN), on the candidates' scale (interior splits halved):
 * an exhaustive query's values measure the proposal's recall */
int oc_topo_result_problems(const oc_topo_result* r, int* nProblems, int* cand, double* ewExact, double* ewPred);
/* per local problem: triangles, free vertices, Newton iterations,
 * line-search energy evaluations and SM clock cycles of its solve (of the
 * one-step pass where the learned proposal did not select it) */
int oc_topo_result_problem_stats(const oc_topo_result* r, int* nProblems, int* nTri, int* nFree, int* iters,
                                 int* trials, long long* cycles);

/* ---- The MLP of the learned proposal (no counterpart in the reference) --
 * in -> hidden -> hidden -> 1 with ReLU; BF16 weights and activations, FP32
 * accumulation; trained on the device (MSE, Adam on FP32 master weights).
 * Parameters: W1 (hidden x in), b1, W2 (hidden x hidden), b2, W3 (hidden), b3. */
int oc_mlp_create(oc_ctx* ctx, int nIn, int nHidden, unsigned seed, oc_mlp** out);
int oc_mlp_destroy(oc_mlp* mlp);
int oc_mlp_num_params(const oc_mlp* mlp, int* n);
int oc_mlp_get_params(oc_mlp* mlp, float* params);
int oc_mlp_set_params(oc_mlp* mlp, const float* params);
int oc_mlp_predict(oc_mlp* mlp, const float* X, int n, float* y);
/* gradient of the mean squared error over n rows (and the loss) */
int oc_mlp_gradient(oc_mlp* mlp, const float* X, const float* target, int n, float* grad, float* loss);
int oc_mlp_train(oc_mlp* mlp, const float* X, const float* target, int n, int epochs, int batch, float lr,
                 unsigned seed, float* finalLoss);
/* the hidden-layer products (K and N >= 16) on the 5th-generation tensor
 * cores (tcgen05.mma, FP32 accumulator in tensor memory; on = 1, the
 * default) or on the CUDA cores (on = 0); OC_ERR_TIMEOUT if a tensor-core
 * wait ran out */
int oc_mlp_set_tensor_cores(oc_mlp* mlp, int on);
/* the network's product on host arrays: C (M x N, row-major) =
 * sum_k A[m*sam + k*sak] B[k*sbk + n*sbn], BF16 operands, FP32 accumulation,
 * on the tensor cores (tensorCores 1) or the CUDA cores (0) */
int oc_bf16_gemm(oc_ctx* ctx, int M, int N, int K, const float* A, long long sam, long long sak, const float* B,
                 long long sbk, long long sbn, float* C, int tensorCores);
/* The bound of the tensor-core kernels' mbarrier waits for later launches,
 * in polls (0: give up at once; -1: the default, 2^20; process-wide).  A
 * wait that runs out ends that product with OC_ERR_TIMEOUT after its MMAs
 * in flight have drained; the context stays usable.  A bound of 0
 * exercises that path. */
int oc_tc_set_wait_polls(int polls);
/* candidate count, index of the largest E_w decrease (-1: none), size of
 * the filtered pool (inSplitTotalAmt for interior splits), local problems
 * solved, their largest iteration count, host build and device solve ms */
int oc_topo_result_info(const oc_topo_result* r, int* nCand, int* best, int* pool, int* nProblems, int* maxIters,
                        double* buildMs, double* solveMs);
/* Newton iterations summed over all local problems, how many of them
 * stopped at the iteration cap (100), and the line-search energy trials */
int oc_topo_result_iterations(const oc_topo_result* r, int* totalIters, int* capped, long long* trials);
/* candidate c as the reference records it: EwDec (interior splits halved,
 * TriMesh.cpp:702-704), energyChanges (2), path (<= 3), newVertPos (<= 4 x 2) */
int oc_topo_result_candidate(const oc_topo_result* r, int c, double* EwDec, double* energyChanges, int* path,
                             int* pathLen, double* newVertPos, int* posRows);
/* all candidates at once: EwDec (nCand), energyChanges (nCand x 2), path
 * (nCand x 3, unused entries -1), newVertPos (nCand x 8, unused 0) and
 * posRows (nCand); NULL arrays are skipped */
int oc_topo_result_candidates(const oc_topo_result* r, double* EwDec, double* energyChanges, int* path,
                              double* newVertPos, int* posRows);
/* bijective queries: local problems with an air loop, those abandoned,
 * the most Steiner points one of their air meshes got, and the problems
 * whose loop refinement stopped at the mesher's limits (0 expected) */
int oc_topo_result_air(const oc_topo_result* r, int* problems, int* rejected, int* steinerMax, int* capped);
int oc_topo_result_destroy(oc_topo_result* r);
/* Optimizer::createFracture(EDecThres, 0, false, splitInterior)
 * (Optimizer.cpp:440-503) -> TriMesh::splitOrMerge (TriMesh.cpp:978-1052):
 * the boundary-split and merge queries (or the interior-split query) on the
 * optimizer's current state with lambda_t = 1 - energyParams[0], the larger
 * E_w decrease (split on ties) applied as oc_optimizer_create_fracture does
 * when it exceeds EDecThres.  With mlp, the queries are the learned
 * proposal's (top fraction topFrac solved exactly).  *changed = 1 when an
 * operation was applied; *opType and *EwDecMax report the best candidate
 * (-DBL_MAX: none). */
int oc_optimizer_split_or_merge(oc_optimizer* opt, double EDecThres, int splitInterior, double filterExp, int options,
                                oc_mlp* mlp, double topFrac, int* changed, int* opType, double* EwDecMax);
/* Optimizer::createFracture(opType, path, newVertPos) (Optimizer.cpp:373-440):
 * applies the operation to the optimizer's mesh (TriMesh::splitEdgeOnBoundary,
 * cutPath or mergeBoundaryEdges with their vertex and cohesive-edge
 * bookkeeping), rebuilds the device mesh and the Newton pattern, rebuilds
 * the scaffold when one is set (the project's generator) and recomputes
 * the energy.  path / newVertPos as a query candidate reports them. */
int oc_optimizer_create_fracture(oc_optimizer* opt, int opType, const int* path, int pathLen,
                                 const double* newVertPos, int posRows);
/* durations (ms) of the last oc_optimizer_create_fracture's phases: host mesh
 * edit, device mesh rebuild, scaffold rebuild, Newton pattern and symbolic
 * analysis (host), their device allocation and upload, energy evaluation */
int oc_optimizer_apply_timing(oc_optimizer* opt, double* out6);
/* The direct solver's last symbolic analysis: carried = the number of
 * carried analyses since the last full one (0: that was a full analysis),
 * host milliseconds of its dissection (0 when carried) and of its front
 * structures, its factor flops and those of the last full analysis. */
int oc_optimizer_analysis_info(oc_optimizer* opt, int* carried, double* ndMs, double* symMs, double* flops,
                               double* fullFlops);
/* the same operation on a mesh alone */
int oc_mesh_apply_topology(oc_mesh* mesh, int opType, const int* path, int pathLen, const double* newVertPos,
                           int posRows);

/* ---- the outer loop's pieces ------------------------------------------
 * Several queries of one state solved together (ops: up to three of
 * OC_OP_*; out: one result per op), as oc_topology_step does for all three;
 * mlp / topFrac select the learned proposal (mlp NULL: exhaustive). */
int oc_topology_queries(oc_mesh* mesh, const int* ops, int nOps, double lambda_t, double filterExp, int options,
                        oc_mlp* mlp, double topFrac, oc_topo_result** out);
/* The local solves' schedule autotuner (queries with OC_TOPO_AUTOTUNE): on
 * the first batch of each (device, size class, problem-count bucket,
 * triangle-count bucket) the class's candidate schedules (threads per
 * problem, block size, cluster size) are timed on the batch itself and the
 * fastest is kept for later batches of that key; without the flag the fixed
 * rule applies, so that the schedule (and the rounding of clustered sums)
 * does not depend on timing.  The table, one row per key: rows (n x 11:
 * device, class (+4 for one-iteration probe passes), log2 count, log2
 * triangles, the chosen tpp / cluster / block, the rule's tpp / cluster /
 * block, candidates timed) and ms (n x 2: chosen, rule). */
int oc_topology_schedules(int* nRows, int* rows, float* ms);
/* The same queries sharded over shardCount processes (one GPU each): the
 * candidate lists are enumerated in full on every shard, but only candidates
 * c with c % shardCount == shardRank get their local solves; the others
 * report EwDec -DBL_MAX and energyChanges (DBL_MAX, DBL_MAX).  Merging the
 * shards' lists (candidate c from shard c % shardCount) gives the unsharded
 * result; the argmax over it is the topology step's choice (one exchange of
 * the lists per step, e.g. an all-gather). */
int oc_topology_queries_sharded(oc_mesh* mesh, const int* ops, int nOps, double lambda_t, double filterExp,
                                int options, oc_mlp* mlp, double topFrac, int shardRank, int shardCount,
                                oc_topo_result** out);
/* querySplit / queryMerge with propagate = true (TriMesh.cpp:637-665,
 * 828-833): OC_OP_BOUNDARY_SPLIT evaluates the boundary splits at the
 * current fracture tail (or at both ends of the last interior split),
 * OC_OP_MERGE the zipper pair forking at the tail. */
int oc_topology_query_tail(oc_mesh* mesh, int opType, double lambda_t, int options, oc_topo_result** out);
/* TriMesh::curFracTail and curInteriorFracTails (-1: none) as the applied
 * operations leave them (TriMesh.cpp:2891-2899, 3046-3048, 3169-3171;
 * Optimizer.cpp:397-399) */
int oc_mesh_fracture_tails(oc_mesh* mesh, int* tails3);
int oc_mesh_set_fracture_tails(oc_mesh* mesh, const int* tails3);
/* TriMesh::computeSeamSparsity (TriMesh.cpp:1542-1558) before the division
 * by virtualRadius: rest length of the interior cohesive edges */
int oc_mesh_seam_length(oc_mesh* mesh, double* seamLen);
/* Optimizer::lastEDec: the last line search's energy decrease */
int oc_optimizer_last_edec(oc_optimizer* opt, double* eDec);
/* Optimizer::setAllowEDecRelTol (Optimizer.cpp:148-151): off, a Newton
 * iteration stops only at the gradient tolerance or a zero step */
int oc_optimizer_set_allow_edec_rel_tol(oc_optimizer* opt, int allow);
/* energyParams[0] as the optimizer holds it */
int oc_optimizer_get_energy_param(oc_optimizer* opt, double* energyParam);
/* Optimizer::setConfig (Optimizer.cpp:287-300): the optimizer's mesh
 * replaced by a recorded state of the same run (same triangle count; rest
 * positions, UV, triangles, cohesive edges, fracture tails or NULL), the
 * scaffold rebuilt when one is set, the energy recomputed and the Newton
 * iteration count set to iterNum. */
int oc_optimizer_set_state(oc_optimizer* opt, int nV, const double* Vrest, const double* UV, int nF, const int* F,
                           int nCohE, const int* cohE, const int* tails3, int iterNum);

/* ---- OptCuts outer loop (src/main.cpp:538-1086 preDrawFunc offline,
 * updateLambda_stationaryV, converge_preDrawFunc) ---------------------------
 * Alternates the inner Newton loop (with fracture propagation after each
 * iteration, Optimizer.cpp:232-262) and the topology step, updates lambda
 * (the dual step) with oscillation detection and best-feasible rollback,
 * and ends at the distortion bound b_d.  It drives an optimizer that
 * precompute has prepared; the mesh carries the cohesive edges of its
 * initial cut (oc_mesh_set_cohesive_edges). */
typedef struct oc_optcuts oc_optcuts;
typedef struct {
    double upperBound;   /* b_d (4.1; values <= 4 become 4.1, main.cpp:1266-1269) */
    int bijective;       /* 1: bijectivity on (main.cpp's bijectiveParam): the
                            optimizer's scaffold (started after the first inner
                            loop when the optimizer has none, main.cpp:991-994)
                            rebuilt after every Newton step and operation, the
                            topology queries in their bijective form
                            (OC_TOPO_BIJECTIVE), no exact final solve */
    int topoLineSearch;  /* 1: fracture propagation after each operation */
    double filterExp;    /* filterExp_in, the interior-split filter (0.6) */
    int topoOptions;     /* OC_TOPO_FP32_HESSIAN */
    oc_mlp* mlp;         /* learned proposal for the queries (NULL: exhaustive) */
    double topFrac;      /* its fraction solved exactly (0.1) */
    int maxNewtonIters;  /* stop (OC_ERR_NOT_CONVERGED) past this many Newton iterations */
    int recordFeatures;  /* 1: keep the (features, target) pairs of every exhaustive
                            topology query (training data for the learned proposal) */
} oc_optcuts_config;
int oc_optcuts_default_config(oc_optcuts_config* cfg);
int oc_optcuts_create(oc_optimizer* opt, oc_mesh* mesh, const oc_optcuts_config* cfg, oc_optcuts** out);
int oc_optcuts_destroy(oc_optcuts* oc);
/* at most maxSteps passes of preDrawFunc; *finished = 1 once the outer loop
 * ended (converge_preDrawFunc, incl. its exact final solve) */
int oc_optcuts_run(oc_optcuts* oc, int maxSteps, int* finished);
/* out[12]: E_SD, E_se (seam length / virtualRadius), lambda, E_w, Newton
 * iterations, topology steps, finished, vertices, and the milliseconds spent
 * in Newton iterations, topology queries, applied operations, in total */
int oc_optcuts_state(oc_optcuts* oc, double* out12);
/* one row per outer event: Newton iterations, E_SD, E_se, lambda,
 * vertices, code (0 inner loop converged, 1 boundary split or merge applied,
 * 2 interior split, 3 interior split after widening the filter, 4/5/6
 * critical-lambda boundary split / interior split / merge, 10 oscillation
 * (rolled back to the best feasible state), 11 converged at the bound,
 * 12 no merge left) */
int oc_optcuts_events(const oc_optcuts* oc, int* nRows, double* rows);
/* one row per Newton iteration: iterations, E_w, E_SD, E_se, lambda,
 * vertices, ||gradient||^2 at the iteration's start */
int oc_optcuts_trace(const oc_optcuts* oc, int* nRows, double* rows);
/* The reference's output files of a run into directory dir (which must
 * exist): energyValPerIter.txt and gradientPerIter.txt
 * (Optimizer::writeEnergyValToFile / writeGradL2NormToFile,
 * Optimizer.cpp:706-740: per Newton iteration E_w, E_SD, E_se/virtualRadius,
 * energyParams[0]; ||g||^2 and the distortion term's own), info.txt
 * (saveInfoForPresent, main.cpp:346-387: sizes, iteration counts, lambda,
 * timings, E_SD and seam length, the four standard stretch measures, the
 * initial seams) and finalResult_mesh.obj (TriMesh::saveAsMesh,
 * TriMesh.cpp:1758-1969).  F0 (nF x 3, the input mesh's triangles, NULL:
 * vertices merged along the cohesive edges) and nV0 give the OBJ's 3D
 * vertex numbering; lambdaInit is info.txt's initial lambda. */
int oc_optcuts_write(oc_optcuts* oc, const char* dir, const int* F0, int nV0, double lambdaInit);
/* the mesh the outer loop edits, and TriMesh::initSeams (the cohesive edges
 * of the initial cut, rows x 4, as the loop started) */
int oc_optcuts_mesh(const oc_optcuts* oc, oc_mesh** mesh);
/* the pairs recorded with recordFeatures: nRows x 32 features and nRows
 * targets (NULL arrays: the count only) */
int oc_optcuts_features(const oc_optcuts* oc, int* nRows, float* X, float* target);
int oc_optcuts_initial_seams(const oc_optcuts* oc, int* nRows, int* rows);
/* TriMesh::saveAsMesh (TriMesh.cpp:1805-1969): rest positions indexed by F0
 * (the input mesh's triangles, nF x 3; NULL: the cut mesh's vertices merged
 * back along the cohesive edges), the current UV as texture coordinates
 * (scaleUV: normalised to the unit square), faces "f v/vt". */
int oc_mesh_write_obj(oc_mesh* mesh, const char* path, const int* F0, int nV0, int scaleUV);
/* the mesh's current topology: counts, and into non-NULL arrays F, V_rest, cohE */
int oc_mesh_get_topology(oc_mesh* mesh, int* nV, int* nF, int* nCohE, int* F, double* Vrest, int* cohE);
/* host only: the operation on plain arrays; outputs hold nV + 2 vertices and
 * nCohE + 2 cohesive rows at most */
int oc_topology_apply(int opType, const int* path, int pathLen, const double* newVertPos, int posRows, int nV, int nF,
                      const int* F, const double* Vrest, const double* UV, int nCohE, const int* cohE, int* F_out,
                      double* Vrest_out, double* UV_out, int* cohE_out, int* nV_out, int* nCohE_out);
/* host only: TriMesh::cutPath(path, makeCoh = true) (TriMesh.cpp:1393-1517) as
 * the initial cutting of a genus >= 1 mesh calls it (main.cpp:1397-1484):
 * from a boundary end every interior edge of the path split on the boundary
 * (cut through where both ends are on the boundary); an interior path first
 * cut through its first three vertices.  Outputs hold nV + 2 * pathLen
 * vertices and nCohE + 2 * pathLen cohesive rows at most; *nSplit (may be
 * NULL) = edges split on the boundary */
int oc_topology_cut_path(const int* path, int pathLen, int nV, int nF, const int* F, const double* Vrest,
                         const double* UV, int nCohE, const int* cohE, int* F_out, double* Vrest_out, double* UV_out,
                         int* cohE_out, int* nV_out, int* nCohE_out, int* nSplit);
/* host only: igl::cut_to_disk as the reference vendors it
 * (src/Utils/cut_to_disk.cpp; called at main.cpp:1429): the cut graph of a
 * genus >= 1 surface, cut i = cutVerts[cutOff[i] .. cutOff[i + 1]) (a closed
 * loop repeats its first vertex).  With cutVerts or cutOff NULL only
 * *nCuts and *nVerts are set; else capCuts >= *nCuts + 1 and
 * capVerts >= *nVerts are required */
int oc_cut_to_disk(const int* F, int nF, int* cutVerts, int capVerts, int* cutOff, int capCuts, int* nCuts,
                   int* nVerts);
/* host only: the split filter's candidate vertices, in order */
int oc_topology_split_candidates(int nV, const int* F, int nF, const double* divGrad, int interior, double filterExp,
                                 int* cands, int* nCands, int* pool);

/* ---- Air mesh without Triangle (replaces Scaffold.cpp:27-205) -----------
 * Host-only.  For a UV layout (UV nV x 2, F nF x 3) and the mesh's rest
 * avgEdgeLen: the boundary loops (each started at its smallest vertex), the
 * reference's segmented bounding box (margin 4 avgEdgeLen, segments about
 * 9 avgEdgeLen) and a constrained Delaunay triangulation of the region
 * between them, every mesh component's interior removed; with
 * minAngleDeg > 0 the air region is refined towards that minimum angle
 * (Triangle's "q" uses 20) by interior Steiner points, never on a segment
 * (as "Y").  Rows of airV: the nBnd boundary vertices (loop by loop), the
 * box points, then the Steiner points.  OC_ERR_INVALID if the boundary
 * self-touches or no boundary exists. */
typedef struct oc_air_mesh oc_air_mesh;
int oc_air_mesh_build(const double* UV, int nV, const int* F, int nF, double avgEdgeLen, double minAngleDeg,
                      oc_air_mesh** out);
int oc_air_mesh_sizes(const oc_air_mesh* am, int* nAirV, int* nAirF, int* nBnd);
int oc_air_mesh_get(const oc_air_mesh* am, double* airV, int* airF, int* bnd);
int oc_air_mesh_destroy(oc_air_mesh* am);
/* The local air loops of the bijective topology solves (Triangle "qYQ" on
 * the loop, Scaffold.cpp:150-170, as the local Scaffold constructor calls
 * it): the region inside the simple polygon pts (nPts x 2, either
 * orientation, 3 <= nPts <= 48) as its constrained Delaunay triangulation,
 * refined towards a 20 degree minimum angle with at most maxSteiner
 * (<= 12) interior Steiner points and none on the polygon.  Host-only; the
 * same code runs inside the bijective local solves.  V (nV x 2: the
 * polygon's points, then the Steiner points; room for nPts + 12 rows) and
 * T (nT x 3, counter-clockwise; room for nPts + 22 rows); status: 0, or 8
 * / 16 when refinement stopped at the Steiner / queue limit. */
int oc_air_loop_mesh(const double* pts, int nPts, int maxSteiner, int* nV, double* V, int* nT, int* T,
                     int* status);

#ifdef __cplusplus
}
#endif
#endif
