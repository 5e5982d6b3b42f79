/* CPU restatement ("port") of the reference OptCuts geometry step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load this library, and only as a checker
 * or as the timed CPU baseline.  The product never links it.
 *
 * Parity pin: every function is checked against golden vectors produced by
 * the reference's own compiled sources (tests/golden/, generated by
 * tests/golden/make_golden.py through oracle/ref/).
 *
 * Layouts: row-major; V_rest nV x 3, UV nV x 2, F nF x 3 (int32),
 * gradient / search direction 2*nV interleaved [u0, v0, u1, v1, ...]
 * (src/Energy/SymDirichletEnergy.cpp:262, src/Optimizer.cpp:666-669).
 * rest: nF x 8 = triArea, triAreaSq, e0SqLen, e1SqLen, e0dote1,
 * e0SqLen_div_dbAreaSq, e1SqLen_div_dbAreaSq, e0dote1_div_dbAreaSq
 * (src/TriMesh.hpp:44-52).
 */
#ifndef OC_ORACLE_H
#define OC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* TriMesh::computeFeatures rest constants (src/TriMesh.cpp:343-404).
 * scalars[0..2] = surfaceArea, avgEdgeLen, virtualRadius. Returns 0, or -1
 * if a rest triangle has zero area (the reference exits there). */
int ocr_rest_constants(const double* V_rest, int nV, const int* F, int nF,
                       double areaThres, double* rest, double* scalars);

/* SymDirichletEnergy::getEnergyValPerElem (SymDirichletEnergy.cpp:24-46). */
void ocr_energy_elem(const double* rest, const int* F, int nF, const double* UV,
                     int uniformWeight, double* out);
/* Energy::computeEnergyVal = sum of the above (Energy.cpp:35-40). */
double ocr_energy(const double* rest, const int* F, int nF, const double* UV, int uniformWeight);

/* SymDirichletEnergy::computeGradient (SymDirichletEnergy.cpp:258-304). */
void ocr_gradient(const double* rest, const int* F, int nF, const double* UV, int nV,
                  const int* fixedVert, int nFixed, int uniformWeight, double* grad);

/* Per-triangle 6x6 Hessian projected to PSD (SymDirichletEnergy.cpp:438-525 +
 * IglUtils::makePD, IglUtils.hpp:71-90); out is nF x 36 row-major, local
 * order (u1, v1, u2, v2, u3, v3).  No fixed-vertex removal, no scaling. */
void ocr_hessian_blocks(const double* rest, const int* F, int nF, const double* UV,
                        int uniformWeight, double* out);

/* SymDirichletEnergy::initStepSize (SymDirichletEnergy.cpp:551-610);
 * lowers *stepSize in place. */
void ocr_init_step_size(const int* F, int nF, const double* UV, const double* dir, double* stepSize);

/* Sparse LDL^T of the assembled Newton matrix and one solve.
 * Pattern: vertex adjacency from F + diagonal; fixed rows are identity*param
 * (LinSysSolver.hpp:37-135, SymDirichletEnergy.cpp:541-548, Optimizer.cpp:825). */
typedef struct ocr_solver ocr_solver;
ocr_solver* ocr_solver_create(int nV, const int* F, int nF, const int* fixedVert, int nFixed,
                              const double* V_rest);
/* Same factorisation under a caller-given vertex elimination order. */
ocr_solver* ocr_solver_create_ordered(int nV, const int* F, int nF, const int* fixedVert, int nFixed,
                                      const int* vertexOrder);
/* Number of negative D entries of the last factorisation. */
int ocr_solver_negative_pivots(const ocr_solver*);
void ocr_solver_destroy(ocr_solver*);
/* blocks: nF x 36 (as from ocr_hessian_blocks), scaled by param; returns 0 or -1 on a non-positive pivot */
int ocr_solver_factorize(ocr_solver*, const double* blocks, double param);
void ocr_solver_solve(ocr_solver*, const double* rhs, double* x);
long long ocr_solver_nnz_L(const ocr_solver*);

/* Whole projected-Newton loop, scaffold off (Optimizer::precompute/solve/
 * solve_oneStep/lineSearch, Optimizer.cpp:154-261, 505-652).
 * UV (in/out) nV x 2.  trace arrays have room for maxIter+1 entries:
 *   traceE[k]      lastEnergyVal after k iterations (traceE[0] = initial)
 *   traceGsq[k]    ||g||^2 at the start of iteration k
 *   traceAlpha[k]  accepted step size of iteration k
 * Returns the number of iterations run; *status = last solve() result (0/1). */
typedef struct {
    double energyParam;   /* energyParams[0] = 1 - lambda */
    double relGL2Tol;     /* Optimizer.cpp:70 (1e-12) */
    int maxIter;
    int nThreads;         /* threads for the per-triangle loops (TBB stand-in) */
} ocr_newton_opts;
int ocr_newton(const double* V_rest, int nV, const int* F, int nF, const int* fixedVert, int nFixed,
               double* UV, const ocr_newton_opts* opts,
               double* traceE, double* traceGsq, double* traceAlpha, double* traceSeconds, int* status);

/* The same loop with the bijectivity scaffold (the scaffolding branches of
 * Optimizer.cpp:764-843 and lineSearch :585-634, Scaffold.cpp:179-293): an
 * air mesh (airV nAirV x 2, airF, bnd as Scaffold's members) given once and
 * moved with every step (Scaffold::stepForward), not rebuilt per iteration.
 * traceE holds energies including the scaffold term. */
typedef struct {
    const double* airV;
    int nAirV;
    const int* airF;
    int nAirF;
    const int* bnd;
    int nBnd;
    double areaThres;     /* areaThres_AM (Scaffold.cpp:189) */
} ocr_scaffold;
int ocr_newton_scaffold(const double* V_rest, int nV, const int* F, int nF, const int* fixedVert, int nFixed,
                        double* UV, const ocr_newton_opts* opts, const ocr_scaffold* scaffold,
                        double* traceE, double* traceGsq, double* traceAlpha, double* traceSeconds, int* status);

/* Topology queries, bijectivity off (oc_topo_oracle.cpp): querySplit
 * (opType 0 boundary, 1 interior) or queryMerge (2) on the state (F, V_rest,
 * UV, cohE), candidates run on nThreads.  Per candidate c < maxCand: EwDec,
 * energyChanges ec[2c..2c+1], path[3c..3c+2] (-1 padded), newVertPos
 * pos[8c..] with posRows[c] rows.  *nCand = number of candidates,
 * *seconds = wall time of the query. */
int ocr_topology_query(int nV, const int* F, int nF, const double* Vrest, const double* UV, const int* cohE,
                       int nCohE, int opType, double lambda_t, double filterExp, int nThreads, int maxCand,
                       double* EwDec, double* ec, int* path, double* pos, int* posRows, int* nCand, double* seconds);

#ifdef __cplusplus
}
#endif
#endif
