// GPU drop-in for the reference's SymDirichletEnergy (src/Energy/
// SymDirichletEnergy.hpp:15-42, the Energy interface of
// src/Energy/Energy.hpp:16-46).  Energy, per-element energy, gradient,
// triplet Hessian (6x6 per triangle, PSD-projected) and the injective step
// bound run in the library; the values are the reference's bit for bit
// (same operation order, FP64).  The device mesh is kept per TriMesh
// topology and its UV refreshed on every call.  Include after the
// reference's SymDirichletEnergy.hpp; link with liboc_gpu.so.
#pragma once

#include "SymDirichletEnergy.hpp"
#include "TriMesh.hpp"
#include "optcuts_gpu.h"

#include <Eigen/Core>

#include <stdexcept>
#include <string>
#include <vector>

namespace OptCuts {

class GpuSymDirichletEnergy : public SymDirichletEnergy {
public:
    explicit GpuSymDirichletEnergy(oc_ctx* ctx) : ctx_(ctx) {}
    ~GpuSymDirichletEnergy() override
    {
        if (mesh_) oc_mesh_destroy(mesh_);
    }

    // Energy::computeEnergyVal (Energy.cpp:35-40)
    void computeEnergyVal(const TriMesh& d, double& E, bool uniform = false) const override
    {
        sync(d);
        check(oc_sd_energy(mesh_, uniform, &E), "computeEnergyVal");
    }
    // SymDirichletEnergy::getEnergyValPerElem (SymDirichletEnergy.cpp:24-46)
    void getEnergyValPerElem(const TriMesh& d, Eigen::VectorXd& e, bool uniform = false) const override
    {
        sync(d);
        e.resize(d.F.rows());
        check(oc_sd_energy_per_elem(mesh_, uniform, e.data()), "getEnergyValPerElem");
    }
    // SymDirichletEnergy::computeGradient (SymDirichletEnergy.cpp:258-304)
    void computeGradient(const TriMesh& d, Eigen::VectorXd& g, bool uniform = false) const override
    {
        sync(d);
        g.resize(2 * d.V.rows());
        check(oc_sd_gradient(mesh_, uniform, g.data()), "computeGradient");
    }
    // SymDirichletEnergy::computeHessian(data, V, I, J) (SymDirichletEnergy.cpp:429-549):
    // per-triangle PSD blocks from the device, appended as the reference's
    // IglUtils::addBlockToMatrix does (free x free entries, triangle order),
    // then the unit diagonal of the fixed vertices (addDiagonalToMatrix)
    void computeHessian(const TriMesh& d, Eigen::VectorXd* V, Eigen::VectorXi* I = NULL, Eigen::VectorXi* J = NULL,
                        bool uniform = false) const override
    {
        sync(d);
        const int nF = static_cast<int>(d.F.rows());
        std::vector<double> blocks(36 * (size_t)nF);
        check(oc_sd_hessian_blocks(mesh_, uniform, blocks.data()), "computeHessian");
        std::vector<double> v;
        std::vector<int> ii, jj;
        for (int t = 0; t < nF; ++t) {
            int idx[3];
            for (int k = 0; k < 3; ++k) idx[k] = d.fixedVert.count(d.F(t, k)) ? -1 : d.F(t, k);
            for (int a = 0; a < 3; ++a) {
                if (idx[a] < 0) continue;
                for (int b = 0; b < 3; ++b) {
                    if (idx[b] < 0) continue;
                    for (int p = 0; p < 2; ++p)
                        for (int q = 0; q < 2; ++q) {
                            v.push_back(blocks[36 * (size_t)t + 6 * (2 * a + p) + 2 * b + q]);
                            ii.push_back(2 * idx[a] + p);
                            jj.push_back(2 * idx[b] + q);
                        }
                }
            }
        }
        for (int f : d.fixedVert)
            for (int p = 0; p < 2; ++p) {
                v.push_back(1.0);
                ii.push_back(2 * f + p);
                jj.push_back(2 * f + p);
            }
        const Eigen::Index base = V->size();
        V->conservativeResize(base + (Eigen::Index)v.size());
        for (size_t k = 0; k < v.size(); ++k) (*V)[base + (Eigen::Index)k] = v[k];
        if (I) {
            I->conservativeResize(base + (Eigen::Index)ii.size());
            J->conservativeResize(base + (Eigen::Index)jj.size());
            for (size_t k = 0; k < ii.size(); ++k) {
                (*I)[base + (Eigen::Index)k] = ii[k];
                (*J)[base + (Eigen::Index)k] = jj[k];
            }
        }
    }
    // the dense form stays the base class's (the small local solves)
    using SymDirichletEnergy::computeHessian;
    // SymDirichletEnergy::initStepSize (SymDirichletEnergy.cpp:551-610): only lowers stepSize
    void initStepSize(const TriMesh& d, const Eigen::VectorXd& dir, double& step) const override
    {
        sync(d);
        check(oc_sd_init_step_size(mesh_, dir.data(), &step), "initStepSize");
    }

private:
    static void check(int rc, const char* what)
    {
        if (rc != OC_OK)
            throw std::runtime_error(std::string("GpuSymDirichletEnergy::") + what + ": " + oc_status_string(rc));
    }
    void sync(const TriMesh& d) const
    {
        using RowMat = Eigen::Matrix<double, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor>;
        RowMat uv = d.V;
        if (!mesh_ || nF_ != d.F.rows() || nV_ != d.V.rows() || F_ != d.F) {
            if (mesh_) oc_mesh_destroy(mesh_);
            mesh_ = nullptr;
            RowMat vr = d.V_rest;
            Eigen::Matrix<int, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor> F = d.F;
            std::vector<int> fixed(d.fixedVert.begin(), d.fixedVert.end());
            check(oc_mesh_create(ctx_, vr.data(), uv.data(), (int)d.V.rows(), F.data(), (int)F.rows(), fixed.data(),
                                 (int)fixed.size(), 0.0, &mesh_),
                  "oc_mesh_create");
            nF_ = d.F.rows();
            nV_ = d.V.rows();
            F_ = d.F;
        }
        else {
            check(oc_mesh_set_uv(mesh_, uv.data()), "oc_mesh_set_uv");
        }
    }
    oc_ctx* ctx_;
    mutable oc_mesh* mesh_ = nullptr;
    mutable Eigen::Index nF_ = -1, nV_ = -1;
    mutable Eigen::MatrixXi F_;
};

} // namespace OptCuts
