// Test driver of the GB300 force plugin through the OpenMM API subset.
//
//   shim_driver describe <input> <output>   SDMForce::describe() of the input system
//   shim_driver evaluate <input> <output>   a Context holding the force: energy, forces and
//                                           results; then lambda1 += 0.1 through
//                                           updateParametersInContext and again
//   shim_driver noneq <input> <output>      the non-equilibrium protocol over nsteps steps of
//                                           dt (context time advanced by hand, two
//                                           evaluations per step time): per step the energy and
//                                           results[SDM_R_RESERVED]; then the work value, the
//                                           work after setNoneqWorkvalue(1.5), and after one
//                                           more step
//   shim_driver rebox <input> <output>      evaluate, evaluate again, change the box and
//                                           evaluate: results[SDM_R_RESERVED], [SDM_R_U0] and
//                                           [SDM_R_U1] after each, getPerturbationEnergy; then a
//                                           triclinic box (an OpenMMException)
//   shim_driver atomic <input> <output>     failed updateParametersInContext calls change nothing
//
// Built with SDM_TEST_CUDA_PLATFORM (and SDMCudaKernels.cpp, CudaSubset.cpp):
//   shim_driver factory - <output>          registerKernelFactories on a CUDA platform: which
//                                           platforms support CalcSDMForce, the kernel created
//                                           by name, an unknown name refused (no GPU needed)
//   shim_driver cuda-mixed|cuda-double <input> <output>
//                                           the evaluate sequence on the CUDA platform (the
//                                           CalcSDMForce kernel on shuffled device arrays), then
//                                           forces without energy and the results read after it
//
// Input (little-endian): int32 n, n_exceptions, method (OpenMM NonbondedMethod),
// dispersion_correction; float64 box[3], cutoff, eps_rf, ewald_tol,
// params[SDM_NPARAMS], charge[n], sigma[n], epsilon[n], displacement[3n],
// positions[3n], exceptions[n_exceptions][5] (i, j, charge product, sigma, epsilon);
// mode noneq only: float64 ntmax, dt; int32 nsteps.
// An OpenMMException prints its message on stderr and exits with status 3.
#include "SDMForceGB300.h"
#include "openmm/Context.h"
#include "openmm/System.h"
#ifdef SDM_TEST_CUDA_PLATFORM
#include "openmm/cuda/CudaPlatform.h"
extern "C" void registerKernelFactories();
#endif

#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

using namespace OpenMM;

namespace {

struct Reader {
    FILE* f;
    template <class T> T one() {
        T v;
        if (fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("short input");
        return v;
    }
    std::vector<double> many(size_t k) {
        std::vector<double> v(k);
        if (k && fread(v.data(), sizeof(double), k, f) != k) throw std::runtime_error("short input");
        return v;
    }
};

template <class T> void put(FILE* f, const T* p, size_t k) { fwrite(p, sizeof(T), k, f); }

#ifdef SDM_TEST_CUDA_PLATFORM
CudaPlatform* cuda_platform(const std::string& precision) {
    static CudaPlatform* cp = nullptr;
    if (!cp) {
        cp = new CudaPlatform(precision);
        Platform::registerPlatform(cp);
        registerKernelFactories();
    }
    return cp;
}

int factory(const char* out_path) {
    CudaPlatform* cp = cuda_platform("mixed");
    FILE* fo = fopen(out_path, "w");
    if (!fo) throw std::runtime_error("cannot open output");
    for (int i = 0; i < Platform::getNumPlatforms(); ++i) {
        Platform& p = Platform::getPlatform(i);
        fprintf(fo, "platform %s supports %d\n", p.getName().c_str(), (int)p.supportsKernels({"CalcSDMForce"}));
    }
    System system;
    system.addParticle(1.0);
    Context context(system, *cp);
    Kernel k = cp->createKernel("CalcSDMForce", context.getImplForTests());
    fprintf(fo, "kernel %s\n", k.getName().c_str());
    try {
        cp->createKernel("NoSuchKernel", context.getImplForTests());
        fprintf(fo, "unknown accepted\n");
    } catch (const OpenMMException& e) {
        fprintf(fo, "unknown refused: %s\n", e.what());
    }
    fclose(fo);
    return 0;
}
#endif

int run(const std::string& mode, const char* in_path, const char* out_path) {
#ifdef SDM_TEST_CUDA_PLATFORM
    if (mode == "factory") return factory(out_path);
#endif
    FILE* fi = fopen(in_path, "rb");
    if (!fi) throw std::runtime_error("cannot open input");
    Reader r{fi};
    const int n = r.one<int>(), nx = r.one<int>(), method = r.one<int>(), disp = r.one<int>();
    std::vector<double> box = r.many(3);
    const double cutoff = r.one<double>(), eps_rf = r.one<double>(), tol = r.one<double>();
    std::vector<double> params = r.many(SDM_NPARAMS), q = r.many(n), sig = r.many(n), eps = r.many(n);
    std::vector<double> d = r.many(3 * (size_t)n), x = r.many(3 * (size_t)n), ex = r.many(5 * (size_t)nx);
    double ntmax = 0.0, dt = 0.0;
    int nsteps = 0;
    if (mode == "noneq") {
        ntmax = r.one<double>();
        dt = r.one<double>();
        nsteps = r.one<int>();
    }
    fclose(fi);

    NonbondedForce nb;
    for (int i = 0; i < n; ++i) nb.addParticle(q[i], sig[i], eps[i]);
    for (int e = 0; e < nx; ++e)
        nb.addException((int)ex[5 * e], (int)ex[5 * e + 1], ex[5 * e + 2], ex[5 * e + 3], ex[5 * e + 4]);
    nb.setNonbondedMethod((NonbondedForce::NonbondedMethod)method);
    nb.setCutoffDistance(cutoff);
    nb.setReactionFieldDielectric(eps_rf);
    nb.setEwaldErrorTolerance(tol);
    nb.setUseDispersionCorrection(disp != 0);

    auto* force = new SDMPluginGB300::SDMForce(nb);
    force->setBiasMethod((int)params[SDM_P_BIAS_METHOD]);
    force->setSoftCoreMethod((int)params[SDM_P_SOFTCORE_METHOD]);
    force->setLambda(params[SDM_P_LAMBDA]);
    force->setLambda1(params[SDM_P_LAMBDA1]);
    force->setLambda2(params[SDM_P_LAMBDA2]);
    force->setAlpha(params[SDM_P_ALPHA]);
    force->setU0(params[SDM_P_U0]);
    force->setW0coeff(params[SDM_P_W0]);
    force->setGamma(params[SDM_P_GAMMA]);
    force->setWBcoeff(params[SDM_P_WB]);
    force->setUmax(params[SDM_P_UMAX]);
    force->setAcore(params[SDM_P_ACORE]);
    force->setUbcore(params[SDM_P_UBCORE]);
    force->setNonEquilibrium((int)params[SDM_P_NONEQ]);
    force->setlambda1Slope(params[SDM_P_M_LAMBDA1]);
    force->setlambda2Slope(params[SDM_P_M_LAMBDA2]);
    force->setu0Slope(params[SDM_P_M_U0]);
    force->setw0Slope(params[SDM_P_M_W0]);
    force->setlambda1intercept(params[SDM_P_B_LAMBDA1]);
    force->setlambda2intercept(params[SDM_P_B_LAMBDA2]);
    force->setu0intercept(params[SDM_P_B_U0]);
    force->setw0intercept(params[SDM_P_B_W0]);
    for (int i = 0; i < n; ++i)
        if (d[3 * i] != 0.0 || d[3 * i + 1] != 0.0 || d[3 * i + 2] != 0.0)
            force->setDisplacement(i, d[3 * i], d[3 * i + 1], d[3 * i + 2]);

    FILE* fo = fopen(out_path, "wb");
    if (!fo) throw std::runtime_error("cannot open output");
    if (mode == "describe") {
        sdm_system_desc s = force->describe(box.data());
        int counts[4] = {s.num_exclusions, s.num_exceptions, s.nonbonded_method, force->getForceGroup()};
        put(fo, counts, 4);
        put(fo, s.exclusions, 2 * (size_t)s.num_exclusions);
        put(fo, s.exception_pairs, 2 * (size_t)s.num_exceptions);
        put(fo, s.exception_params, 3 * (size_t)s.num_exceptions);
        put(fo, s.displacement, 3 * (size_t)n);
        const double scal[4] = {s.cutoff, s.reaction_field_dielectric, s.ewald_tolerance, s.box[0] + s.box[1] + s.box[2]};
        put(fo, scal, 4);
        put(fo, force->getParameterBlock(), SDM_NPARAMS);
        fclose(fo);
        delete force;
        return 0;
    }
    System system;
    for (int i = 0; i < n; ++i) system.addParticle(12.0);
    system.setDefaultPeriodicBoxVectors(Vec3(box[0], 0, 0), Vec3(0, box[1], 0), Vec3(0, 0, box[2]));
    system.addForce(force);
    std::vector<Vec3> pos(n);
    for (int i = 0; i < n; ++i) pos[i] = Vec3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
#ifdef SDM_TEST_CUDA_PLATFORM
    const bool on_cuda = mode == "cuda-mixed" || mode == "cuda-double";
    Context context = on_cuda ? Context(system, *cuda_platform(mode == "cuda-double" ? "double" : "mixed"))
                              : Context(system);
#else
    const bool on_cuda = false;
    Context context(system);
#endif
    context.setPositions(pos);
    if (mode == "rebox") {
        for (int k = 0; k < 3; ++k) {
            if (k == 2) context.setPeriodicBoxVectors(Vec3(box[0] + 0.1, 0, 0), Vec3(0, box[1], 0), Vec3(0, 0, box[2]));
            context.getState(State::Energy, false, 1 << 2);
            const std::vector<double> res = force->getResults(context);
            const double v[3] = {res[SDM_R_RESERVED], res[SDM_R_U0], res[SDM_R_U1]};
            put(fo, v, 3);
        }
        double pe[5];
        force->getPerturbationEnergy(context, pe[0], pe[1], pe[2], pe[3], pe[4]);
        put(fo, pe, 5);
        fclose(fo);
        context.setPeriodicBoxVectors(Vec3(box[0], 0, 0), Vec3(0.5, box[1], 0), Vec3(0, 0, box[2]));
        context.getState(State::Energy, false, 1 << 2);   // throws: the box must be rectangular
        return 0;
    }
    if (mode == "atomic") {
        // a failed updateParametersInContext leaves the context's parameters
        // and displacements as they were, also for a handle re-created later
        auto energy = [&]() { return context.getState(State::Energy, false, 1 << 2).getPotentialEnergy(); };
        double v[6];
        v[0] = energy();
        const double lam = force->getLambda();
        int threw = 0;
        force->setLambda(lam + 0.1);
        force->setDisplacement(0, std::nan(""), 0.0, 0.0);   // refused by the force before any push
        try { force->updateParametersInContext(context); } catch (const OpenMMException&) { threw |= 1; }
        v[1] = energy();
        force->setDisplacement(0, 2.0e6, 0.0, 0.0);          // refused by the library after the parameters
        force->setLambda(lam + 0.2);
        try { force->updateParametersInContext(context); } catch (const OpenMMException&) { threw |= 2; }
        v[2] = energy();
        context.setPeriodicBoxVectors(Vec3(box[0] + 0.1, 0, 0), Vec3(0, box[1], 0), Vec3(0, 0, box[2]));
        v[3] = energy();   // a new handle, made from what the context holds
        v[4] = force->getResults(context)[SDM_R_U1];
        v[5] = threw;
        put(fo, v, 6);
        fclose(fo);
        return 0;
    }
    if (mode == "noneq") {
        force->setNonEquilibrium(1);
        force->setNoneqtmax(ntmax);
        force->updateParametersInContext(context);
        double t = 0.0;
        auto step = [&]() {
            context.setTime(t);
            double e = 0.0, calls = 0.0;
            for (int rep = 0; rep < 2; ++rep) {   // a second evaluation at the same time adds no work
                e = context.getState(State::Energy, false, 1 << 2).getPotentialEnergy();
                calls = force->getResults(context)[SDM_R_RESERVED];
            }
            put(fo, &e, 1);
            put(fo, &calls, 1);
            t += dt;
        };
        for (int k = 0; k < nsteps; ++k) step();
        context.setTime(t);
        const double w1 = force->getNoneqWorkvalue(context);
        force->setNoneqWorkvalue(context, 1.5);
        const double w2 = force->getNoneqWorkvalue(context);
        step();
        context.setTime(t);
        const double w3 = force->getNoneqWorkvalue(context);
        const double ws[3] = {w1, w2, w3};
        put(fo, ws, 3);
        fclose(fo);
        return 0;
    }
    if (on_cuda) {
        // forces without the energy (the kernel's asynchronous form), then the
        // results of that evaluation read afterwards
        State st = context.getState(State::Forces, false, 1 << 2);
        for (const Vec3& f : st.getForces()) {
            const double v[3] = {f[0], f[1], f[2]};
            put(fo, v, 3);
        }
        std::vector<double> res = force->getResults(context);
        put(fo, res.data(), res.size());
    }
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            force->setLambda1(force->getLambda1() + 0.1);
            force->updateParametersInContext(context);
        }
        State st = context.getState(State::Energy | State::Forces, false, 1 << 2);
        const double e = st.getPotentialEnergy();
        std::vector<double> res = force->getResults(context);
        put(fo, &e, 1);
        put(fo, res.data(), res.size());
        for (const Vec3& f : st.getForces()) {
            const double v[3] = {f[0], f[1], f[2]};
            put(fo, v, 3);
        }
    }
    fclose(fo);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: shim_driver describe|evaluate|noneq|rebox|atomic|factory|cuda-mixed|cuda-double "
                        "<input> <output>\n");
        return 2;
    }
    try {
        return run(argv[1], argv[2], argv[3]);
    } catch (const OpenMMException& e) {
        fprintf(stderr, "%s\n", e.what());
        return 3;
    }
}
