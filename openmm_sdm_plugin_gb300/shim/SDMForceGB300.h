/*
 * SDMForceGB300.h -- OpenMM force plugin over the GB300 SDM two-state force
 * (libsdm_gb300.so, include/sdm_capi.h).
 *
 * The reference drives the SDM method from its integrator: every step of
 * LangevinIntegratorSDM (openmmapi/src/LangevinIntegratorSDM.cpp:153-183)
 * evaluates the group-2 NonbondedForce at x and at x+d, combines the two
 * states in IntegrateLangevinStepSDMKernel::execute
 * (platforms/reference/src/ReferenceSDMKernels.cpp:202-341) and takes a
 * stochastic-dynamics step on the hybrid force (1-s) F0 + s F1 plus the
 * group-1 forces.
 *
 * SDMPluginGB300::SDMForce re-expresses that integrator as a force: it takes
 * the place of the group-2 NonbondedForce and returns E_pot = U0 + W(u') with
 * the hybrid force, evaluated by one sdm_evaluate call.  OpenMM's own
 * LangevinIntegrator then integrates group 1 + this force, which is the
 * reference's step (the reference's ReferenceStochasticDynamicsSDM.cpp:131-266
 * is OpenMM's leap-frog Langevin update).  The SDM parameters carry the
 * setter names of the reference integrator
 * (openmmapi/include/LangevinIntegratorSDM.h); getBindE / getPotEnergy read
 * the last evaluation of a context, as the reference integrator's getters
 * (LangevinIntegratorSDM.h:301-324) read its last step.
 *
 * The implementation derives from OpenMM's CustomCPPForceImpl (OpenMM 8.0 or
 * later): positions arrive in host memory in the System's particle order and
 * forces go back the same way, on every OpenMM platform.
 */
#ifndef SDM_FORCE_GB300_H
#define SDM_FORCE_GB300_H

#include "openmm/Force.h"
#include "openmm/NonbondedForce.h"
#include "openmm/Vec3.h"
#include "sdm_capi.h"

#include <vector>

namespace OpenMM {
class Context;
}

namespace SDMPluginGB300 {

class SDMForce : public OpenMM::Force {
public:
    /* Method ids of the reference integrator (LangevinIntegratorSDM.h:120-122, :143-145). */
    enum BiasMethod { LinearMethod = SDM_LINEAR, QuadraticMethod = SDM_QUADRATIC, ILogisticMethod = SDM_ILOGISTIC };
    enum SoftCoreMethod {
        NoSoftCoreMethod = SDM_NO_SOFTCORE,
        TanhMethod = SDM_TANH_SOFTCORE,
        RationalMethod = SDM_RATIONAL_SOFTCORE
    };

    /* Copies the particles, exceptions, cutoff and electrostatics of `nb`
     * (CutoffPeriodic = reaction field, or PME; no dispersion correction, no
     * switching function) and puts the force in group 2.  `device` is the CUDA
     * device index of the evaluation.  Defaults of the SDM parameters are the
     * reference integrator's constructor defaults (LangevinIntegratorSDM.cpp:58-75). */
    explicit SDMForce(const OpenMM::NonbondedForce& nb, int device = 0);

    /* Parameters (reference setters, LangevinIntegratorSDM.h:75-463). */
    void setLambda(double v) { p_[SDM_P_LAMBDA] = v; }
    double getLambda() const { return p_[SDM_P_LAMBDA]; }
    void setBiasMethod(int m) { p_[SDM_P_BIAS_METHOD] = m; }
    int getBiasMethod() const { return (int)p_[SDM_P_BIAS_METHOD]; }
    void setSoftCoreMethod(int m) { p_[SDM_P_SOFTCORE_METHOD] = m; }
    int getSoftCoreMethod() const { return (int)p_[SDM_P_SOFTCORE_METHOD]; }
    void setGamma(double v) { p_[SDM_P_GAMMA] = v; }
    double getGamma() const { return p_[SDM_P_GAMMA]; }
    void setWBcoeff(double v) { p_[SDM_P_WB] = v; }
    double getWBcoeff() const { return p_[SDM_P_WB]; }
    void setW0coeff(double v) { p_[SDM_P_W0] = v; }
    double getW0coeff() const { return p_[SDM_P_W0]; }
    void setLambda1(double v) { p_[SDM_P_LAMBDA1] = v; }
    double getLambda1() const { return p_[SDM_P_LAMBDA1]; }
    void setLambda2(double v) { p_[SDM_P_LAMBDA2] = v; }
    double getLambda2() const { return p_[SDM_P_LAMBDA2]; }
    void setAlpha(double v) { p_[SDM_P_ALPHA] = v; }
    double getAlpha() const { return p_[SDM_P_ALPHA]; }
    void setU0(double v) { p_[SDM_P_U0] = v; }
    double getU0() const { return p_[SDM_P_U0]; }
    void setUmax(double v) { p_[SDM_P_UMAX] = v; }
    double getUmax() const { return p_[SDM_P_UMAX]; }
    void setAcore(double v) { p_[SDM_P_ACORE] = v; }
    double getAcore() const { return p_[SDM_P_ACORE]; }
    void setUbcore(double v) { p_[SDM_P_UBCORE] = v; }
    double getUbcore() const { return p_[SDM_P_UBCORE]; }
    void setNonEquilibrium(int v) { p_[SDM_P_NONEQ] = v; }
    int getNonEquilibrium() const { return (int)p_[SDM_P_NONEQ]; }
    /* Non-equilibrium protocol (ReferenceSDMKernels.cpp:229-245, 289-302):
     * with setNonEquilibrium(1) and Ntmax > 0 every evaluation uses
     * lambda = t / Ntmax, t the context time, and the context accumulates
     * the work sum over steps of (dt / Ntmax) dW/dlambda at the step start. */
    void setNoneqtmax(double t) { ntmax_ = t; }
    double getNoneqtmax() const { return ntmax_; }
    double getNoneqWorkvalue(OpenMM::Context& context);
    void setNoneqWorkvalue(OpenMM::Context& context, double work);
    void setlambda1Slope(double v) { p_[SDM_P_M_LAMBDA1] = v; }
    double getlambda1Slope() const { return p_[SDM_P_M_LAMBDA1]; }
    void setlambda2Slope(double v) { p_[SDM_P_M_LAMBDA2] = v; }
    double getlambda2Slope() const { return p_[SDM_P_M_LAMBDA2]; }
    void setu0Slope(double v) { p_[SDM_P_M_U0] = v; }
    double getu0Slope() const { return p_[SDM_P_M_U0]; }
    void setw0Slope(double v) { p_[SDM_P_M_W0] = v; }
    double getw0Slope() const { return p_[SDM_P_M_W0]; }
    void setlambda1intercept(double v) { p_[SDM_P_B_LAMBDA1] = v; }
    double getlambda1intercept() const { return p_[SDM_P_B_LAMBDA1]; }
    void setlambda2intercept(double v) { p_[SDM_P_B_LAMBDA2] = v; }
    double getlambda2intercept() const { return p_[SDM_P_B_LAMBDA2]; }
    void setu0intercept(double v) { p_[SDM_P_B_U0] = v; }
    double getu0intercept() const { return p_[SDM_P_B_U0]; }
    void setw0intercept(double v) { p_[SDM_P_B_W0] = v; }
    double getw0intercept() const { return p_[SDM_P_B_W0]; }
    void setDisplacement(int atom, double dx, double dy, double dz);
    OpenMM::Vec3 getDisplacement(int atom) const;

    int getNumParticles() const { return (int)charge_.size(); }
    const double* getParameterBlock() const { return p_; }

    /* Pushes the SDM parameters and the displacements to a context that
     * already holds this force (as OpenMM forces' updateParametersInContext). */
    void updateParametersInContext(OpenMM::Context& context);

    /* Results of the context's last evaluation, SDM_NRESULTS doubles in the
     * order of sdm_capi.h (U0, U1, u, u', ..., E_pot, dW/dlambda, ...). */
    std::vector<double> getResults(OpenMM::Context& context);
    double getBindE(OpenMM::Context& context) { return getResults(context)[SDM_R_BINDE]; }
    /* U0 + W: the reference's getPotEnergy() without the group-1 energy. */
    double getPotEnergy(OpenMM::Context& context) { return getResults(context)[SDM_R_EPOT]; }
    /* u, U0, U1, W and W' of the context's last evaluation. */
    void getPerturbationEnergy(OpenMM::Context& context, double& u, double& u0, double& u1, double& w, double& dw) {
        const std::vector<double> r = getResults(context);
        u = r[SDM_R_U];
        u0 = r[SDM_R_U0];
        u1 = r[SDM_R_U1];
        w = r[SDM_R_W];
        dw = r[SDM_R_DW];
    }

    /* The system descriptor handed to sdm_create for a box (a, b, c diagonal);
     * the pointers stay valid while this force lives and is not modified. */
    sdm_system_desc describe(const double box[3]) const;

    bool usesPeriodicBoundaryConditions() const override { return true; }

protected:
    OpenMM::ForceImpl* createImpl() const override;

private:
    friend class SDMForceImpl;
    friend class SDMContextState;
    int device_;
    double p_[SDM_NPARAMS];
    std::vector<double> charge_, sigma_, epsilon_, displ_;
    std::vector<int> exclusions_, exception_pairs_;
    std::vector<double> exception_params_;
    double cutoff_, eps_rf_, ewald_tol_;
    int method_;
    int pme_grid_[3];
    double ntmax_ = 0.0;
};

}  // namespace SDMPluginGB300

#endif
