/*
 * SDMCudaKernels.cpp -- CalcSDMForce on OpenMM's CUDA platform, its kernel
 * factory and the plugin entry points OpenMM calls when it loads the
 * library (registerPlatforms / registerKernelFactories, the pair the
 * reference exports at platforms/reference/src/ReferenceSDMKernelFactory.cpp:41-56
 * and platforms/opencl/src/OpenCLSDMKernelFactory.cpp:39-61).
 *
 * The kernel keeps the two-state force on the device.  Each execute() is one
 * sdm_evaluate_engine call on OpenMM-CUDA's current stream: it gathers the
 * reordered positions (posq, plus posqCorrection in mixed precision) through
 * the atom index, evaluates both states with the combine, and adds the hybrid
 * force into OpenMM-CUDA's 64-bit fixed-point force buffer (2^32 scale,
 * component-major, paddedNumAtoms stride) -- the arrays the reference's
 * OpenCL kernels save, displace, restore and mix in place
 * (platforms/opencl/src/OpenCLSDMKernels.cpp:104-146, 271-276).  Positions
 * and forces never cross the host link.  The results (U0, U1, u, W, W', ...)
 * come back to the host only when OpenMM asks for the energy, when the
 * non-equilibrium protocol needs dW/dlambda, and every kStatusInterval
 * evaluations, when the device status word is checked.
 *
 * The handle is made on OpenMM's device (CudaContext::getDeviceIndex) and
 * uses the CUDA runtime there, that is the device's primary context, which
 * is the context OpenMM 8's CUDA platform runs in.
 */
#include "SDMKernels.h"

#include "openmm/OpenMMException.h"
#include "openmm/cuda/CudaContext.h"
#include "openmm/cuda/CudaPlatform.h"
#include "openmm/internal/ContextImpl.h"

#include <memory>
#include <string>

namespace SDMPluginGB300 {

using OpenMM::OpenMMException;

namespace {

void check(sdm_status st, const sdm_handle* h, const char* what) {
    if (st != SDM_OK)
        throw OpenMMException(std::string("SDMForce: ") + what + ": " + sdm_last_error(h));
}

// evaluations between two reads of the device status word when nothing
// else synchronises (a list overflow then shows within this many steps)
constexpr int kStatusInterval = 64;

class CudaCalcSDMForceKernel : public CalcSDMForceKernel {
public:
    CudaCalcSDMForceKernel(std::string name, const OpenMM::Platform& platform, OpenMM::CudaContext& cu)
        : CalcSDMForceKernel(name, platform), cu_(cu) {}

    void initialize(const OpenMM::System& system, const SDMForce& force) override {
        st_.reset(new SDMContextState(force));
        st_->setDevice(cu_.getDeviceIndex());
        st_->initialize(system);
    }

    double execute(OpenMM::ContextImpl& context, bool includeForces, bool includeEnergy) override {
        sdm_handle* h = st_->prepare(context);
        const bool sync = includeEnergy || st_->nonEquilibrium() || ++calls_ % kStatusInterval == 0;
        void* corr = cu_.getUseMixedPrecision() ? (void*)cu_.getPosqCorrection().getDevicePointer() : nullptr;
        check(sdm_evaluate_engine(h, (const void*)cu_.getPosq().getDevicePointer(), corr,
                                  cu_.getUseDoublePrecision() ? 1 : 0,
                                  (const int*)cu_.getAtomIndexArray().getDevicePointer(), cu_.getPaddedNumAtoms(),
                                  includeForces ? (long long*)cu_.getLongForceBuffer().getDevicePointer() : nullptr,
                                  sync ? st_->results() : nullptr, (void*)cu_.getCurrentStream()),
              h, "evaluation failed");
        stale_ = !sync;
        if (sync) st_->finish(context);
        return includeEnergy ? st_->results()[SDM_R_EPOT] : 0.0;
    }

    void copyParametersToContext(OpenMM::ContextImpl& context, const SDMForce& force) override { st_->update(force); }

    const double* getResults() override {
        if (stale_ && st_->handle()) {
            check(sdm_get_last_results(st_->handle(), st_->results()), st_->handle(), "reading the results failed");
            stale_ = false;
        }
        return st_->results();
    }

    void getPerturbationEnergy(double& u, double& u0, double& u1, double& w, double& dw) override {
        const double* r = getResults();
        u = r[SDM_R_U];
        u0 = r[SDM_R_U0];
        u1 = r[SDM_R_U1];
        w = r[SDM_R_W];
        dw = r[SDM_R_DW];
    }

    double getNoneqWorkvalue(const OpenMM::ContextImpl& context) override { return st_->work(context); }
    void setNoneqWorkvalue(const OpenMM::ContextImpl& context, double work) override { st_->setWork(context, work); }

private:
    OpenMM::CudaContext& cu_;
    std::unique_ptr<SDMContextState> st_;
    long long calls_ = 0;
    bool stale_ = false;
};

class CudaSDMKernelFactory : public OpenMM::KernelFactory {
public:
    OpenMM::KernelImpl* createKernelImpl(std::string name, const OpenMM::Platform& platform,
                                         OpenMM::ContextImpl& context) const override {
        OpenMM::CudaPlatform::PlatformData& data =
            *static_cast<OpenMM::CudaPlatform::PlatformData*>(context.getPlatformData());
        if (name == CalcSDMForceKernel::Name()) return new CudaCalcSDMForceKernel(name, platform, *data.contexts[0]);
        throw OpenMMException("Tried to create kernel with illegal kernel name '" + name + "'");
    }
};

}  // namespace

}  // namespace SDMPluginGB300

extern "C" OPENMM_EXPORT void registerPlatforms() {}

/* Registers the CalcSDMForce factory with OpenMM's CUDA platform, when that
 * platform is loaded; other platforms keep SDMForce's host path. */
extern "C" OPENMM_EXPORT void registerKernelFactories() {
    for (int i = 0; i < OpenMM::Platform::getNumPlatforms(); ++i) {
        OpenMM::Platform& platform = OpenMM::Platform::getPlatform(i);
        if (platform.getName() == "CUDA")
            platform.registerKernelFactory(SDMPluginGB300::CalcSDMForceKernel::Name(),
                                           new SDMPluginGB300::CudaSDMKernelFactory());
    }
}

extern "C" OPENMM_EXPORT void registerSDMGB300CudaKernelFactories() { registerKernelFactories(); }
