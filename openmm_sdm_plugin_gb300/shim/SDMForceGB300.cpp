/*
 * SDMForceGB300.cpp -- the OpenMM force plugin over libsdm_gb300.so.
 *
 * SDMForce copies what the reference reads from the group-2 NonbondedForce
 * (the particles and exceptions that example/desmonddmsfile75.py:772-850
 * puts there, the cutoff and the electrostatics of :418-426).  SDMForceImpl
 * owns one sdm_handle per context: initialize() is the reference kernel's
 * initialize (platforms/reference/src/ReferenceSDMKernels.cpp:144-159), and
 * computeForce() is one step's two group-2 evaluations, the state save,
 * displace and restore (LangevinIntegratorSDM.cpp:158-173) and the combine
 * of ReferenceSDMKernels.cpp:231-318, in one sdm_evaluate call.
 */
#include "SDMForceGB300.h"
#include "SDMKernels.h"

#include "openmm/Context.h"
#include "openmm/OpenMMException.h"
#include "openmm/internal/ContextImpl.h"
#include "openmm/internal/CustomCPPForceImpl.h"

#include <cmath>
#include <string>

namespace SDMPluginGB300 {

using OpenMM::OpenMMException;
using OpenMM::Vec3;

namespace {

void check(sdm_status st, const sdm_handle* h, const char* what) {
    if (st != SDM_OK)
        throw OpenMMException(std::string("SDMForce: ") + what + ": " + sdm_last_error(h));
}

}  // namespace

SDMForce::SDMForce(const OpenMM::NonbondedForce& nb, int device) : device_(device) {
    using OpenMM::NonbondedForce;
    const int n = nb.getNumParticles();
    charge_.resize(n);
    sigma_.resize(n);
    epsilon_.resize(n);
    for (int i = 0; i < n; ++i) nb.getParticleParameters(i, charge_[i], sigma_[i], epsilon_[i]);
    displ_.assign(3 * (size_t)n, 0.0);
    // every exception is an excluded pair; the ones with a charge product or
    // a well depth interact with their own parameters (the 1-4 pairs)
    for (int e = 0; e < nb.getNumExceptions(); ++e) {
        int i, j;
        double qq, sg, ep;
        nb.getExceptionParameters(e, i, j, qq, sg, ep);
        exclusions_.push_back(i);
        exclusions_.push_back(j);
        if (qq != 0.0 || ep != 0.0) {
            exception_pairs_.push_back(i);
            exception_pairs_.push_back(j);
            exception_params_.push_back(qq);
            exception_params_.push_back(sg);
            exception_params_.push_back(ep);
        }
    }
    cutoff_ = nb.getCutoffDistance();
    eps_rf_ = nb.getReactionFieldDielectric();
    ewald_tol_ = nb.getEwaldErrorTolerance();
    pme_grid_[0] = pme_grid_[1] = pme_grid_[2] = 0;
    switch (nb.getNonbondedMethod()) {
        case NonbondedForce::CutoffPeriodic: method_ = SDM_NB_REACTION_FIELD; break;
        case NonbondedForce::PME: {
            method_ = SDM_NB_PME;
            double alpha;
            int nx, ny, nz;
            nb.getPMEParameters(alpha, nx, ny, nz);
            // the library derives the splitting parameter from the tolerance
            // (OpenMM's rule); an explicit alpha would be a different model
            if (alpha != 0.0)
                throw OpenMMException("SDMForce: explicit PME parameters are not supported; "
                                      "set the Ewald error tolerance instead");
            break;
        }
        default:
            throw OpenMMException("SDMForce: the NonbondedForce must use CutoffPeriodic (reaction field) or PME");
    }
    if (nb.getUseDispersionCorrection())
        throw OpenMMException("SDMForce: the NonbondedForce must have setUseDispersionCorrection(false)");
    if (nb.getUseSwitchingFunction())
        throw OpenMMException("SDMForce: switching functions are not supported");
    // reference integrator defaults (LangevinIntegratorSDM.cpp:56-75)
    for (double& v : p_) v = 0.0;
    p_[SDM_P_BIAS_METHOD] = LinearMethod;
    p_[SDM_P_SOFTCORE_METHOD] = NoSoftCoreMethod;
    p_[SDM_P_LAMBDA] = 1.0;
    p_[SDM_P_WB] = 1.0;
    p_[SDM_P_LAMBDA1] = 1.0;
    p_[SDM_P_LAMBDA2] = 1.0;
    p_[SDM_P_ALPHA] = 1.0;
    p_[SDM_P_UMAX] = 200.0;
    p_[SDM_P_ACORE] = 0.25;
    setForceGroup(2);
}

void SDMForce::setDisplacement(int atom, double dx, double dy, double dz) {
    if (atom < 0 || atom >= getNumParticles()) throw OpenMMException("SDMForce: particle index out of range");
    displ_[3 * (size_t)atom + 0] = dx;
    displ_[3 * (size_t)atom + 1] = dy;
    displ_[3 * (size_t)atom + 2] = dz;
}

Vec3 SDMForce::getDisplacement(int atom) const {
    if (atom < 0 || atom >= getNumParticles()) throw OpenMMException("SDMForce: particle index out of range");
    const double* d = &displ_[3 * (size_t)atom];
    return Vec3(d[0], d[1], d[2]);
}

sdm_system_desc SDMForce::describe(const double box[3]) const {
    sdm_system_desc d = {};
    d.num_particles = getNumParticles();
    d.charge = charge_.data();
    d.sigma = sigma_.data();
    d.epsilon = epsilon_.data();
    d.num_exclusions = (int)(exclusions_.size() / 2);
    d.exclusions = exclusions_.data();
    d.displacement = displ_.data();
    for (int k = 0; k < 3; ++k) d.box[k] = box[k];
    d.cutoff = cutoff_;
    d.reaction_field_dielectric = eps_rf_;
    d.num_replicas = 1;
    d.num_exceptions = (int)(exception_params_.size() / 3);
    d.exception_pairs = exception_pairs_.data();
    d.exception_params = exception_params_.data();
    d.nonbonded_method = method_;
    d.ewald_tolerance = ewald_tol_;
    for (int k = 0; k < 3; ++k) d.pme_grid[k] = pme_grid_[k];
    return d;
}

// ---------------------------------------------------------------------------
// SDMContextState: one context's handle, parameters and work bookkeeping
// ---------------------------------------------------------------------------
SDMContextState::SDMContextState(const SDMForce& owner) : owner_(owner) {
    for (double& v : res_) v = 0.0;
    for (double& v : p_) v = 0.0;
}

SDMContextState::~SDMContextState() { sdm_destroy(h_); }

void SDMContextState::boxOf(OpenMM::ContextImpl& context, double box[3]) {
    Vec3 a, b, c;
    context.getPeriodicBoxVectors(a, b, c);
    if (a[1] != 0.0 || a[2] != 0.0 || b[0] != 0.0 || b[2] != 0.0 || c[0] != 0.0 || c[1] != 0.0)
        throw OpenMMException("SDMForce: the periodic box must be rectangular");
    box[0] = a[0];
    box[1] = b[1];
    box[2] = c[2];
}

void SDMContextState::initialize(const OpenMM::System& system) {
    if (system.getNumParticles() != owner_.getNumParticles())
        throw OpenMMException("SDMForce: particle count differs from the System's");
    for (int k = 0; k < SDM_NPARAMS; ++k) p_[k] = owner_.p_[k];
    ntmax_ = owner_.ntmax_;
    displ_ = owner_.displ_;
}

/* One sdm_handle per context.  The box is fixed at handle creation; a
 * context whose box changes (a barostat) gets a new handle. */
void SDMContextState::create(OpenMM::ContextImpl& context) {
    boxOf(context, box_);
    sdm_destroy(h_);
    h_ = nullptr;
    sdm_system_desc d = owner_.describe(box_);
    d.displacement = displ_.data();
    check(sdm_create(&d, 1, device_ >= 0 ? device_ : owner_.device_, &h_), nullptr, "sdm_create failed");
    check(sdm_set_params(h_, 0, p_), h_, "invalid SDM parameters");
}

sdm_handle* SDMContextState::prepare(OpenMM::ContextImpl& context) {
    double box[3];
    boxOf(context, box);
    if (!h_ || box[0] != box_[0] || box[1] != box_[1] || box[2] != box_[2]) create(context);
    if (nonEquilibrium()) {
        const double t = context.getTime();
        // the step from the last evaluation's time to t is complete: its
        // work increment uses dW/dlambda at that step's start
        if (have_last_ && t != t_last_) work_ += (t - t_last_) / ntmax_ * dwdl_last_;
        const double lam = t / ntmax_;
        if (lam != p_[SDM_P_LAMBDA]) {
            p_[SDM_P_LAMBDA] = lam;
            check(sdm_set_params(h_, 0, p_), h_, "invalid SDM parameters");
        }
    }
    return h_;
}

void SDMContextState::finish(OpenMM::ContextImpl& context) {
    if (!nonEquilibrium()) return;
    have_last_ = true;
    t_last_ = context.getTime();
    dwdl_last_ = res_[SDM_R_DWDLAMBDA];
}

/* All or nothing: on any error the handle and this object keep the
 * parameters and displacements of the last successful update, so a later
 * re-creation (box change) applies consistent values. */
void SDMContextState::update(const SDMForce& f) {
    if (f.displ_.size() != displ_.size())
        throw OpenMMException("SDMForce: the displacement map must keep the particle count");
    for (double v : f.displ_)
        if (!std::isfinite(v)) throw OpenMMException("SDMForce: invalid displacement: non-finite value");
    check(sdm_set_params(h_, 0, f.p_), h_, "invalid SDM parameters");
    const sdm_status st = sdm_set_displacement(h_, 0, f.displ_.data());
    if (st != SDM_OK) {
        const std::string msg = std::string("invalid displacement: ") + sdm_last_error(h_);
        sdm_set_params(h_, 0, p_);   // back to the parameters that this object still holds
        throw OpenMMException("SDMForce: " + msg);
    }
    for (int k = 0; k < SDM_NPARAMS; ++k) p_[k] = f.p_[k];
    ntmax_ = f.ntmax_;
    displ_ = f.displ_;
}

/* The accumulated work plus the increment of the step that ends at the
 * context's current time (its force evaluation at the step start is the
 * last one seen). */
double SDMContextState::work(const OpenMM::ContextImpl& context) const {
    if (!have_last_ || !(ntmax_ > 0.0)) return work_;
    return work_ + (context.getTime() - t_last_) / ntmax_ * dwdl_last_;
}

void SDMContextState::setWork(const OpenMM::ContextImpl& context, double w) { work_ += w - work(context); }

// ---------------------------------------------------------------------------
// SDMForceImpl: the platform kernel where a factory provides one (OpenMM's
// CUDA platform with this plugin's kernels registered), else the host path
// ---------------------------------------------------------------------------
class SDMForceImpl : public OpenMM::CustomCPPForceImpl {
public:
    explicit SDMForceImpl(const SDMForce& owner) : OpenMM::CustomCPPForceImpl(owner), owner_(owner), st_(owner) {}

    void initialize(OpenMM::ContextImpl& context) override {
        OpenMM::Platform& platform = context.getPlatform();
        if (platform.supportsKernels({CalcSDMForceKernel::Name()})) {
            kernel_ = platform.createKernel(CalcSDMForceKernel::Name(), context);
            kernel_.getAs<CalcSDMForceKernel>().initialize(context.getSystem(), owner_);
            have_kernel_ = true;
            return;
        }
        OpenMM::CustomCPPForceImpl::initialize(context);
        st_.initialize(context.getSystem());
        st_.prepare(context);   // the handle now: a bad descriptor fails the context's creation
    }

    bool usesKernel() const { return have_kernel_; }

    double calcForcesAndEnergy(OpenMM::ContextImpl& context, bool includeForces, bool includeEnergy,
                               int groups) override {
        if (!usesKernel()) return OpenMM::CustomCPPForceImpl::calcForcesAndEnergy(context, includeForces, includeEnergy, groups);
        if ((groups & (1 << owner_.getForceGroup())) == 0) return 0.0;
        return kernel_.getAs<CalcSDMForceKernel>().execute(context, includeForces, includeEnergy);
    }

    double computeForce(OpenMM::ContextImpl& context, const std::vector<Vec3>& positions,
                        std::vector<Vec3>& forces) override {
        sdm_handle* h = st_.prepare(context);
        const size_t n = positions.size();
        x_.resize(3 * n);
        f_.resize(3 * n);
        for (size_t i = 0; i < n; ++i) {
            x_[3 * i + 0] = positions[i][0];
            x_[3 * i + 1] = positions[i][1];
            x_[3 * i + 2] = positions[i][2];
        }
        double* res = st_.results();
        check(sdm_evaluate(h, x_.data(), res, f_.data()), h, "evaluation failed");
        st_.finish(context);
        forces.resize(n);
        for (size_t i = 0; i < n; ++i) forces[i] = Vec3(f_[3 * i + 0], f_[3 * i + 1], f_[3 * i + 2]);
        return res[SDM_R_EPOT];
    }

    void updateParametersInContext(OpenMM::ContextImpl& context, const SDMForce& f) {
        if (usesKernel()) kernel_.getAs<CalcSDMForceKernel>().copyParametersToContext(context, f);
        else st_.update(f);
    }

    const double* results() {
        return usesKernel() ? kernel_.getAs<CalcSDMForceKernel>().getResults() : st_.results();
    }
    double work(const OpenMM::ContextImpl& context) {
        return usesKernel() ? kernel_.getAs<CalcSDMForceKernel>().getNoneqWorkvalue(context) : st_.work(context);
    }
    void setWork(const OpenMM::ContextImpl& context, double w) {
        if (usesKernel()) kernel_.getAs<CalcSDMForceKernel>().setNoneqWorkvalue(context, w);
        else st_.setWork(context, w);
    }

private:
    const SDMForce& owner_;
    SDMContextState st_;     // the host path's state (the kernel keeps its own)
    OpenMM::Kernel kernel_;
    bool have_kernel_ = false;
    std::vector<double> x_, f_;
};

OpenMM::ForceImpl* SDMForce::createImpl() const { return new SDMForceImpl(*this); }

void SDMForce::updateParametersInContext(OpenMM::Context& context) {
    dynamic_cast<SDMForceImpl&>(getImplInContext(context)).updateParametersInContext(getContextImpl(context), *this);
}

double SDMForce::getNoneqWorkvalue(OpenMM::Context& context) {
    return dynamic_cast<SDMForceImpl&>(getImplInContext(context)).work(getContextImpl(context));
}

void SDMForce::setNoneqWorkvalue(OpenMM::Context& context, double work) {
    dynamic_cast<SDMForceImpl&>(getImplInContext(context)).setWork(getContextImpl(context), work);
}

std::vector<double> SDMForce::getResults(OpenMM::Context& context) {
    const double* r = dynamic_cast<SDMForceImpl&>(getImplInContext(context)).results();
    return std::vector<double>(r, r + SDM_NRESULTS);
}

}  // namespace SDMPluginGB300
