/*
 * Declarations of the subset of OpenMM's public C++ API (OpenMM 8) that the
 * GB300 force plugin (openmm_sdm_plugin_gb300/shim) uses, with minimal
 * bodies, so that the plugin compiles and runs in tests without OpenMM.
 * Class and method names and signatures are OpenMM's; the bodies are
 * single-context stand-ins (one System, positions in host memory, forces
 * summed per group), not OpenMM's implementation.
 */
#ifndef OPENMM_API_SUBSET_H
#define OPENMM_API_SUBSET_H

#include <exception>
#include <map>
#include <string>
#include <vector>

#ifndef OPENMM_EXPORT
#define OPENMM_EXPORT __attribute__((visibility("default")))
#endif

namespace OpenMM {

class Vec3 {
public:
    Vec3() : d{0.0, 0.0, 0.0} {}
    Vec3(double x, double y, double z) : d{x, y, z} {}
    double operator[](int k) const { return d[k]; }
    double& operator[](int k) { return d[k]; }
    Vec3 operator+(const Vec3& o) const { return Vec3(d[0] + o.d[0], d[1] + o.d[1], d[2] + o.d[2]); }

private:
    double d[3];
};

class OpenMMException : public std::exception {
public:
    explicit OpenMMException(const std::string& message) : message(message) {}
    const char* what() const noexcept override { return message.c_str(); }

private:
    std::string message;
};

class Context;
class ContextImpl;
class ForceImpl;
class Platform;

class KernelImpl {
public:
    KernelImpl(std::string name, const Platform& platform) : name(name), platform(&platform) {}
    virtual ~KernelImpl() {}
    std::string getName() const { return name; }
    const Platform& getPlatform() { return *platform; }

private:
    std::string name;
    const Platform* platform;
};

/* A shared handle of a KernelImpl (the last copy deletes it). */
class Kernel {
public:
    Kernel() : impl(nullptr), refs(nullptr) {}
    explicit Kernel(KernelImpl* impl) : impl(impl), refs(new int(1)) {}
    Kernel(const Kernel& o) : impl(o.impl), refs(o.refs) { if (refs) ++*refs; }
    Kernel& operator=(const Kernel& o);
    ~Kernel() { release(); }
    std::string getName() const { return impl->getName(); }
    const KernelImpl& getImpl() const { return *impl; }
    KernelImpl& getImpl() { return *impl; }
    template <class T> T& getAs() { return dynamic_cast<T&>(*impl); }

private:
    void release();
    KernelImpl* impl;
    int* refs;
};

class KernelFactory {
public:
    virtual ~KernelFactory() {}
    virtual KernelImpl* createKernelImpl(std::string name, const Platform& platform, ContextImpl& context) const = 0;
};

class Platform {
public:
    virtual ~Platform();
    virtual const std::string& getName() const = 0;
    void registerKernelFactory(const std::string& name, KernelFactory* factory);
    bool supportsKernels(const std::vector<std::string>& kernelNames) const;
    Kernel createKernel(const std::string& name, ContextImpl& context) const;
    static void registerPlatform(Platform* platform);
    static int getNumPlatforms();
    static Platform& getPlatform(int index);
    static Platform& getPlatformByName(const std::string& name);
    // stand-in hooks (not OpenMM API): platform data of a new context, and
    // the moves of positions and forces between the host and the platform
    virtual void contextCreated(ContextImpl& context) const {}
    virtual void contextDestroyed(ContextImpl& context) const {}
    virtual void positionsChanged(ContextImpl& context) const {}
    virtual void beginForces(ContextImpl& context) const {}
    virtual void endForces(ContextImpl& context) const {}

private:
    std::map<std::string, KernelFactory*> factories;
};

/* The default platform of this subset: host positions, host forces. */
class ReferencePlatform : public Platform {
public:
    const std::string& getName() const override;
};

class Force {
public:
    Force() : forceGroup(0) {}
    virtual ~Force() {}
    int getForceGroup() const { return forceGroup; }
    void setForceGroup(int group) { forceGroup = group; }
    virtual bool usesPeriodicBoundaryConditions() const { return false; }

protected:
    friend class ContextImpl;
    virtual ForceImpl* createImpl() const = 0;
    ForceImpl& getImplInContext(Context& context);
    const ForceImpl& getImplInContext(const Context& context) const;
    ContextImpl& getContextImpl(Context& context);

private:
    int forceGroup;
};

class ForceImpl {
public:
    virtual ~ForceImpl() {}
    virtual void initialize(ContextImpl& context) = 0;
    virtual const Force& getOwner() const = 0;
    virtual void updateContextState(ContextImpl& context, bool& forcesInvalid) = 0;
    virtual double calcForcesAndEnergy(ContextImpl& context, bool includeForces, bool includeEnergy,
                                       int groups) = 0;
    virtual std::map<std::string, double> getDefaultParameters() = 0;
    virtual std::vector<std::string> getKernelNames() = 0;
};

/* Host-side force implementation: computeForce gets the positions and
 * returns the forces in host memory, in the System's particle order. */
class CustomCPPForceImpl : public ForceImpl {
public:
    explicit CustomCPPForceImpl(const Force& owner) : owner(owner) {}
    void initialize(ContextImpl& context) override {}
    virtual double computeForce(ContextImpl& context, const std::vector<Vec3>& positions,
                                std::vector<Vec3>& forces) = 0;
    const Force& getOwner() const override { return owner; }
    void updateContextState(ContextImpl& context, bool& forcesInvalid) override {}
    double calcForcesAndEnergy(ContextImpl& context, bool includeForces, bool includeEnergy, int groups) override;
    std::map<std::string, double> getDefaultParameters() override { return {}; }
    std::vector<std::string> getKernelNames() override { return {}; }

private:
    const Force& owner;
    std::vector<Vec3> forces;
};

class NonbondedForce : public Force {
public:
    enum NonbondedMethod { NoCutoff = 0, CutoffNonPeriodic = 1, CutoffPeriodic = 2, Ewald = 3, PME = 4, LJPME = 5 };
    int getNumParticles() const { return (int)particles.size(); }
    int getNumExceptions() const { return (int)exceptions.size(); }
    int addParticle(double charge, double sigma, double epsilon);
    void getParticleParameters(int index, double& charge, double& sigma, double& epsilon) const;
    int addException(int particle1, int particle2, double chargeProd, double sigma, double epsilon,
                     bool replace = false);
    void getExceptionParameters(int index, int& particle1, int& particle2, double& chargeProd, double& sigma,
                                double& epsilon) const;
    NonbondedMethod getNonbondedMethod() const { return method; }
    void setNonbondedMethod(NonbondedMethod m) { method = m; }
    double getCutoffDistance() const { return cutoff; }
    void setCutoffDistance(double distance) { cutoff = distance; }
    double getReactionFieldDielectric() const { return rfDielectric; }
    void setReactionFieldDielectric(double dielectric) { rfDielectric = dielectric; }
    double getEwaldErrorTolerance() const { return ewaldTol; }
    void setEwaldErrorTolerance(double tol) { ewaldTol = tol; }
    void getPMEParameters(double& alpha, int& nx, int& ny, int& nz) const;
    void setPMEParameters(double alpha, int nx, int ny, int nz);
    bool getUseDispersionCorrection() const { return dispersionCorrection; }
    void setUseDispersionCorrection(bool use) { dispersionCorrection = use; }
    bool getUseSwitchingFunction() const { return switching; }
    void setUseSwitchingFunction(bool use) { switching = use; }
    bool usesPeriodicBoundaryConditions() const override { return method >= CutoffPeriodic; }

protected:
    ForceImpl* createImpl() const override;

private:
    struct Particle { double q, sig, eps; };
    struct Exception { int i, j; double qq, sig, eps; };
    std::vector<Particle> particles;
    std::vector<Exception> exceptions;
    NonbondedMethod method = NoCutoff;
    double cutoff = 1.0, rfDielectric = 78.3, ewaldTol = 5e-4, alpha = 0.0;
    int nx = 0, ny = 0, nz = 0;
    bool dispersionCorrection = true, switching = false;
};

class System {
public:
    ~System();
    int addParticle(double mass) { masses.push_back(mass); return (int)masses.size() - 1; }
    int getNumParticles() const { return (int)masses.size(); }
    double getParticleMass(int index) const { return masses.at(index); }
    int addForce(Force* force) { forces.push_back(force); return (int)forces.size() - 1; }
    int getNumForces() const { return (int)forces.size(); }
    Force& getForce(int index) { return *forces.at(index); }
    const Force& getForce(int index) const { return *forces.at(index); }
    void setDefaultPeriodicBoxVectors(const Vec3& a, const Vec3& b, const Vec3& c) { box[0] = a; box[1] = b; box[2] = c; }
    void getDefaultPeriodicBoxVectors(Vec3& a, Vec3& b, Vec3& c) const { a = box[0]; b = box[1]; c = box[2]; }

private:
    std::vector<double> masses;
    std::vector<Force*> forces;
    Vec3 box[3] = {Vec3(2, 0, 0), Vec3(0, 2, 0), Vec3(0, 0, 2)};
};

class State {
public:
    enum DataType { Positions = 1, Velocities = 2, Forces = 4, Energy = 8 };
    double getPotentialEnergy() const { return energy; }
    const std::vector<Vec3>& getForces() const { return forces; }

private:
    friend class Context;
    double energy = 0.0;
    std::vector<Vec3> forces;
};

class ContextImpl {
public:
    ContextImpl(Context& owner, const System& system, Platform& platform);
    ~ContextImpl();
    const System& getSystem() const { return system; }
    Context& getOwner() { return owner; }
    void getPositions(std::vector<Vec3>& out) { out = positions; }
    void setPositions(const std::vector<Vec3>& p) { positions = p; platform.positionsChanged(*this); }
    void getPeriodicBoxVectors(Vec3& a, Vec3& b, Vec3& c) { a = box[0]; b = box[1]; c = box[2]; }
    void setPeriodicBoxVectors(const Vec3& a, const Vec3& b, const Vec3& c) { box[0] = a; box[1] = b; box[2] = c; }
    double getTime() const { return time; }
    void setTime(double t) { time = t; }
    Platform& getPlatform() { return platform; }
    void* getPlatformData() { return platformData; }
    void setPlatformData(void* data) { platformData = data; }
    std::vector<ForceImpl*>& getForceImpls() { return forceImpls; }
    double calcForcesAndEnergy(bool includeForces, bool includeEnergy, int groups = 0xFFFFFFFF);
    std::vector<Vec3>& getForceAccumulator() { return forces; }

private:
    Context& owner;
    const System& system;
    Platform& platform;
    void* platformData = nullptr;
    std::vector<ForceImpl*> forceImpls;
    std::vector<Vec3> positions, forces;
    Vec3 box[3];
    double time = 0.0;
};

/* A context without an integrator: enough to evaluate forces and energies. */
class Context {
public:
    explicit Context(const System& system);
    Context(const System& system, Platform& platform);
    ~Context();
    // stand-in accessor (not OpenMM API) for tests of kernel factories
    ContextImpl& getImplForTests() { return *impl; }
    void setPositions(const std::vector<Vec3>& positions) { impl->setPositions(positions); }
    void setPeriodicBoxVectors(const Vec3& a, const Vec3& b, const Vec3& c) { impl->setPeriodicBoxVectors(a, b, c); }
    void setTime(double time) { impl->setTime(time); }
    State getState(int types, bool enforcePeriodicBox = false, int groups = 0xFFFFFFFF);

private:
    friend class Force;
    void create(const System& system, Platform& platform);
    ContextImpl* impl;
};

}  // namespace OpenMM

#endif
