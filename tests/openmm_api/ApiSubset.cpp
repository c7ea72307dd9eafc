// Bodies of the OpenMM API subset declared in openmm/ApiSubset.h (test
// stand-ins for one context, not OpenMM's implementation).
#include "openmm/ApiSubset.h"

namespace OpenMM {

ForceImpl& Force::getImplInContext(Context& context) {
    for (ForceImpl* f : context.impl->getForceImpls())
        if (&f->getOwner() == this) return *f;
    throw OpenMMException("getImplInContext: this Force is not present in the Context");
}

const ForceImpl& Force::getImplInContext(const Context& context) const {
    for (ForceImpl* f : context.impl->getForceImpls())
        if (&f->getOwner() == this) return *f;
    throw OpenMMException("getImplInContext: this Force is not present in the Context");
}

ContextImpl& Force::getContextImpl(Context& context) { return *context.impl; }

double CustomCPPForceImpl::calcForcesAndEnergy(ContextImpl& context, bool includeForces, bool includeEnergy,
                                               int groups) {
    if ((groups & (1 << owner.getForceGroup())) == 0) return 0.0;
    std::vector<Vec3> positions;
    context.getPositions(positions);
    double energy = computeForce(context, positions, forces);
    if (includeForces) {
        std::vector<Vec3>& acc = context.getForceAccumulator();
        for (size_t i = 0; i < acc.size() && i < forces.size(); ++i) acc[i] = acc[i] + forces[i];
    }
    return includeEnergy ? energy : 0.0;
}

int NonbondedForce::addParticle(double charge, double sigma, double epsilon) {
    particles.push_back({charge, sigma, epsilon});
    return (int)particles.size() - 1;
}

void NonbondedForce::getParticleParameters(int index, double& charge, double& sigma, double& epsilon) const {
    const Particle& p = particles.at(index);
    charge = p.q;
    sigma = p.sig;
    epsilon = p.eps;
}

int NonbondedForce::addException(int particle1, int particle2, double chargeProd, double sigma, double epsilon,
                                 bool) {
    exceptions.push_back({particle1, particle2, chargeProd, sigma, epsilon});
    return (int)exceptions.size() - 1;
}

void NonbondedForce::getExceptionParameters(int index, int& particle1, int& particle2, double& chargeProd,
                                            double& sigma, double& epsilon) const {
    const Exception& e = exceptions.at(index);
    particle1 = e.i;
    particle2 = e.j;
    chargeProd = e.qq;
    sigma = e.sig;
    epsilon = e.eps;
}

void NonbondedForce::getPMEParameters(double& a, int& x, int& y, int& z) const {
    a = alpha;
    x = nx;
    y = ny;
    z = nz;
}

void NonbondedForce::setPMEParameters(double a, int x, int y, int z) {
    alpha = a;
    nx = x;
    ny = y;
    nz = z;
}

ForceImpl* NonbondedForce::createImpl() const {
    throw OpenMMException("NonbondedForce is not evaluated by this API subset");
}

System::~System() {
    for (Force* f : forces) delete f;
}

void Kernel::release() {
    if (refs && --*refs == 0) {
        delete impl;
        delete refs;
    }
    impl = nullptr;
    refs = nullptr;
}

Kernel& Kernel::operator=(const Kernel& o) {
    if (this != &o) {
        release();
        impl = o.impl;
        refs = o.refs;
        if (refs) ++*refs;
    }
    return *this;
}

namespace {
std::vector<Platform*>& platforms() {
    static std::vector<Platform*> list;
    return list;
}
}  // namespace

Platform::~Platform() {
    for (auto& kv : factories) {
        bool seen = false;   // one factory may serve several names
        for (auto& kv2 : factories) {
            if (&kv2 == &kv) break;
            if (kv2.second == kv.second) seen = true;
        }
        if (!seen) delete kv.second;
    }
}

void Platform::registerKernelFactory(const std::string& name, KernelFactory* factory) { factories[name] = factory; }

bool Platform::supportsKernels(const std::vector<std::string>& kernelNames) const {
    for (const std::string& n : kernelNames)
        if (factories.find(n) == factories.end()) return false;
    return true;
}

Kernel Platform::createKernel(const std::string& name, ContextImpl& context) const {
    auto it = factories.find(name);
    if (it == factories.end())
        throw OpenMMException("Called createKernel() on a Platform which does not support the requested kernel");
    return Kernel(it->second->createKernelImpl(name, *this, context));
}

void Platform::registerPlatform(Platform* platform) { platforms().push_back(platform); }
int Platform::getNumPlatforms() { return (int)platforms().size(); }
Platform& Platform::getPlatform(int index) { return *platforms().at(index); }

Platform& Platform::getPlatformByName(const std::string& name) {
    for (Platform* p : platforms())
        if (p->getName() == name) return *p;
    throw OpenMMException("There is no registered Platform called \"" + name + "\"");
}

const std::string& ReferencePlatform::getName() const {
    static const std::string name = "Reference";
    return name;
}

namespace {
// the default platform, registered when the library loads
struct RegisterReference {
    RegisterReference() { Platform::registerPlatform(new ReferencePlatform()); }
} registerReference;
}  // namespace

ContextImpl::ContextImpl(Context& owner, const System& system, Platform& platform)
    : owner(owner), system(system), platform(platform) {
    system.getDefaultPeriodicBoxVectors(box[0], box[1], box[2]);
    positions.assign(system.getNumParticles(), Vec3());
    platform.contextCreated(*this);
    for (int i = 0; i < system.getNumForces(); ++i) forceImpls.push_back(system.getForce(i).createImpl());
}

ContextImpl::~ContextImpl() {
    for (ForceImpl* f : forceImpls) delete f;
    platform.contextDestroyed(*this);
}

double ContextImpl::calcForcesAndEnergy(bool includeForces, bool includeEnergy, int groups) {
    forces.assign(system.getNumParticles(), Vec3());
    platform.beginForces(*this);
    double energy = 0.0;
    for (ForceImpl* f : forceImpls) energy += f->calcForcesAndEnergy(*this, includeForces, includeEnergy, groups);
    platform.endForces(*this);
    return energy;
}

void Context::create(const System& system, Platform& platform) {
    impl = new ContextImpl(*this, system, platform);
    try {
        for (ForceImpl* f : impl->getForceImpls()) f->initialize(*impl);
    } catch (...) {
        delete impl;
        throw;
    }
}

Context::Context(const System& system) : impl(nullptr) { create(system, Platform::getPlatformByName("Reference")); }

Context::Context(const System& system, Platform& platform) : impl(nullptr) { create(system, platform); }

Context::~Context() { delete impl; }

State Context::getState(int types, bool, int groups) {
    State s;
    const bool wantForces = (types & State::Forces) != 0, wantEnergy = (types & State::Energy) != 0;
    s.energy = impl->calcForcesAndEnergy(wantForces, wantEnergy, groups);
    if (wantForces) s.forces = impl->getForceAccumulator();
    return s;
}

}  // namespace OpenMM
