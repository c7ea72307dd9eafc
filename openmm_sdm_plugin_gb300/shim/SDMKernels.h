/*
 * SDMKernels.h -- the platform-kernel half of the OpenMM plugin.
 *
 * The reference registers one platform kernel, IntegrateLangevinStepSDM
 * (openmmapi/include/SDMKernels.h:47-113), created by its kernel factories
 * (platforms/reference/src/ReferenceSDMKernelFactory.cpp:41-63,
 * platforms/opencl/src/OpenCLSDMKernelFactory.cpp:39-76), which the
 * integrator drives around two NonbondedForce evaluations.  Here the
 * two-state force is one kernel, CalcSDMForce, driven by SDMForce's
 * implementation:
 *
 *   initialize(system, force)            the reference kernel's initialize
 *                                        (ReferenceSDMKernels.cpp:144-159)
 *   execute(context, forces, energy)     both group-2 evaluations, the state
 *                                        copies and the combine of one step
 *                                        (LangevinIntegratorSDM.cpp:158-176,
 *                                        ReferenceSDMKernels.cpp:202-318)
 *   copyParametersToContext(context, f)  updateParametersInContext
 *   getPerturbationEnergy(u, U0, U1, W, W')
 *
 * The CUDA platform's factory (SDMCudaKernels.cpp) creates a kernel that
 * reads OpenMM-CUDA's reordered positions and adds into its 64-bit
 * fixed-point force buffer on the device.  Other platforms keep the host
 * path of CustomCPPForceImpl.
 *
 * SDMContextState is what both paths share: the C-ABI handle of one context,
 * the parameters and displacements it holds, the box it was made for, and
 * the non-equilibrium work bookkeeping.
 */
#ifndef SDM_KERNELS_GB300_H
#define SDM_KERNELS_GB300_H

#include "SDMForceGB300.h"
#include "openmm/KernelImpl.h"
#include "openmm/Platform.h"
#include "openmm/System.h"
#include "openmm/internal/ContextImpl.h"

#include <string>
#include <vector>

namespace SDMPluginGB300 {

class SDMContextState {
public:
    explicit SDMContextState(const SDMForce& owner);
    ~SDMContextState();
    SDMContextState(const SDMContextState&) = delete;
    SDMContextState& operator=(const SDMContextState&) = delete;

    /* Takes the owner's parameters and displacements (a System of the
     * owner's particle count); the handle is made by the first prepare(). */
    void initialize(const OpenMM::System& system);
    /* Before an evaluation at the context's time: a handle for the context's
     * box (made on first use and again when the box changed), the
     * non-equilibrium lambda = t / Ntmax.  Returns the handle. */
    sdm_handle* prepare(OpenMM::ContextImpl& context);
    /* After an evaluation whose results are in results(): the work of the
     * step that ended at the context's time. */
    void finish(OpenMM::ContextImpl& context);
    /* updateParametersInContext: all or nothing. */
    void update(const SDMForce& f);
    double work(const OpenMM::ContextImpl& context) const;
    void setWork(const OpenMM::ContextImpl& context, double w);
    bool nonEquilibrium() const { return p_[SDM_P_NONEQ] == 1.0 && ntmax_ > 0.0; }
    double* results() { return res_; }
    sdm_handle* handle() const { return h_; }
    /* The CUDA device of the handle (default: the force's device). */
    void setDevice(int device) { device_ = device; }

    static void boxOf(OpenMM::ContextImpl& context, double box[3]);

private:
    void create(OpenMM::ContextImpl& context);

    const SDMForce& owner_;
    sdm_handle* h_ = nullptr;
    int device_ = -1;
    double box_[3] = {0.0, 0.0, 0.0};
    double p_[SDM_NPARAMS];
    double res_[SDM_NRESULTS];
    std::vector<double> displ_;
    // non-equilibrium work: the sum over completed steps, and the time and
    // dW/dlambda of the last evaluation
    double ntmax_ = 0.0, work_ = 0.0, t_last_ = 0.0, dwdl_last_ = 0.0;
    bool have_last_ = false;
};

class CalcSDMForceKernel : public OpenMM::KernelImpl {
public:
    static std::string Name() { return "CalcSDMForce"; }
    CalcSDMForceKernel(std::string name, const OpenMM::Platform& platform) : OpenMM::KernelImpl(name, platform) {}
    virtual void initialize(const OpenMM::System& system, const SDMForce& force) = 0;
    /* E_pot = U0 + W of the context's current positions when includeEnergy,
     * else 0; the hybrid force goes into the platform's force buffer. */
    virtual double execute(OpenMM::ContextImpl& context, bool includeForces, bool includeEnergy) = 0;
    virtual void copyParametersToContext(OpenMM::ContextImpl& context, const SDMForce& force) = 0;
    virtual void getPerturbationEnergy(double& u, double& u0, double& u1, double& w, double& dw) = 0;
    /* SDM_NRESULTS doubles of the last evaluation. */
    virtual const double* getResults() = 0;
    virtual double getNoneqWorkvalue(const OpenMM::ContextImpl& context) = 0;
    virtual void setNoneqWorkvalue(const OpenMM::ContextImpl& context, double work) = 0;
};

}  // namespace SDMPluginGB300

#endif
