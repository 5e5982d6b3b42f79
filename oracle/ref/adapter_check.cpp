// Compile-and-link check of the reference-side adapters
// (optcuts_gb300/adapters/): instantiates the energy and linear-solver
// drop-ins against the reference's own headers.  Test infrastructure only;
// linked into oracle/_ref/ref_driver_gpu together with the GPU Optimizer
// (optcuts_gb300/adapters/GpuOptimizer.cpp), which replaces the reference's
// Optimizer.o under the reference's own headless driver.
#include "GpuLinSysSolver.hpp"
#include "GpuSymDirichletEnergy.hpp"

#include <memory>

// never called by the driver: it only makes the compiler build every
// member of the adapters
extern "C" void oc_adapters_instantiate(oc_ctx* ctx)
{
    std::unique_ptr<OptCuts::Energy> e(new OptCuts::GpuSymDirichletEnergy(ctx));
    std::unique_ptr<OptCuts::LinSysSolver<Eigen::VectorXi, Eigen::VectorXd>> ls(
        new OptCuts::GpuLinSysSolver<Eigen::VectorXi, Eigen::VectorXd>(ctx));
    (void)e;
    (void)ls;
}
