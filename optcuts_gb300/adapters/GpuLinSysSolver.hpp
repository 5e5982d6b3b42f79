// GPU drop-in for the reference's LinSysSolver<VectorXi, VectorXd>
// (src/LinSysSolver/LinSysSolver.hpp:22-256).  The matrix lives on the
// device as a full-symmetric 2x2-block CSR over vertices; factorize is the
// library's multifrontal LDL^T (the exact solve SimplicialLDLT performs in
// EigenLibSolver.cpp:79-93), solve its substitutions.  Include after the
// reference's LinSysSolver.hpp; link with liboc_gpu.so.
#pragma once

#include "LinSysSolver.hpp"
#include "optcuts_gpu.h"

#include <Eigen/Sparse>

#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace OptCuts {

template <typename vectorTypeI, typename vectorTypeS>
class GpuLinSysSolver : public LinSysSolver<vectorTypeI, vectorTypeS> {
public:
    explicit GpuLinSysSolver(oc_ctx* ctx)
    {
        check(oc_linsys_create(ctx, &ls_), "oc_linsys_create");
        check(oc_linsys_set_type(ls_, OC_SOLVER_DIRECT), "set_type");
    }
    ~GpuLinSysSolver() override { oc_linsys_destroy(ls_); }

    // threads and matrix type do not apply: the solve is an LDL^T on the device
    void set_type(int, int, bool = false) override {}

    // LinSysSolver::set_pattern(vNeighbor, fixedVert) (LinSysSolver.hpp:37-135),
    // what Optimizer::precompute / updateEnergyData / solve_oneStep call
    // (Optimizer.cpp:174, 358, 524)
    void set_pattern(const std::vector<std::set<int>>& vNeighbor, const std::set<int>& fixedVert) override
    {
        std::vector<int> ptr(1, 0), idx, fixed(fixedVert.begin(), fixedVert.end());
        for (const auto& nb : vNeighbor) {
            idx.insert(idx.end(), nb.begin(), nb.end());
            ptr.push_back(static_cast<int>(idx.size()));
        }
        nV_ = static_cast<int>(vNeighbor.size());
        this->numRows = 2 * nV_;
        check(oc_linsys_set_pattern_neighbors(ls_, nV_, ptr.data(), idx.data(), fixed.data(),
                                              static_cast<int>(fixed.size())),
              "set_pattern");
    }

    // the pattern of an SPD matrix over interleaved (u, v) unknowns
    void set_pattern(const Eigen::SparseMatrix<double>& mtr) override
    {
        nV_ = static_cast<int>(mtr.rows() / 2);
        std::vector<std::set<int>> nb(nV_);
        for (int k = 0; k < mtr.outerSize(); ++k)
            for (Eigen::SparseMatrix<double>::InnerIterator it(mtr, k); it; ++it)
                if (it.row() / 2 != it.col() / 2) nb[it.row() / 2].insert(static_cast<int>(it.col() / 2));
        set_pattern(nb, std::set<int>());
        update_a(mtr);
    }

    // LinSysSolver::update_a(I, J, V) (LinSysSolver.hpp:138-159): i <= j kept
    void update_a(const vectorTypeI& II, const vectorTypeI& JJ, const vectorTypeS& SS) override
    {
        check(oc_linsys_update_a(ls_, II.data(), JJ.data(), SS.data(), static_cast<int>(SS.size())), "update_a");
    }
    void update_a(const Eigen::SparseMatrix<double>& mtr) override
    {
        std::vector<int> I, J;
        std::vector<double> V;
        for (int k = 0; k < mtr.outerSize(); ++k)
            for (Eigen::SparseMatrix<double>::InnerIterator it(mtr, k); it; ++it) {
                I.push_back(static_cast<int>(it.row()));
                J.push_back(static_cast<int>(it.col()));
                V.push_back(it.value());
            }
        check(oc_linsys_update_a(ls_, I.data(), J.data(), V.data(), static_cast<int>(V.size())), "update_a");
    }

    void analyze_pattern(void) override { check(oc_linsys_analyze_pattern(ls_), "analyze_pattern"); }

    // false on a zero or non-finite pivot (EigenLibSolver.cpp:79-93)
    bool factorize(void) override { return oc_linsys_factorize(ls_) == OC_OK; }

    void solve(Eigen::VectorXd& rhs, Eigen::VectorXd& result) override
    {
        result.resize(2 * nV_);
        check(oc_linsys_solve(ls_, rhs.data(), result.data(), 0.0, 0, nullptr, nullptr), "solve");
    }

    void multiply(const Eigen::VectorXd& x, Eigen::VectorXd& Ax) override
    {
        Ax.resize(2 * nV_);
        check(oc_linsys_multiply(ls_, x.data(), Ax.data()), "multiply");
    }

    oc_linsys* handle() const { return ls_; }

private:
    static void check(int rc, const char* what)
    {
        if (rc != OC_OK) throw std::runtime_error(std::string("GpuLinSysSolver::") + what + ": " + oc_status_string(rc));
    }
    oc_linsys* ls_ = nullptr;
    int nV_ = 0;
};

} // namespace OptCuts
