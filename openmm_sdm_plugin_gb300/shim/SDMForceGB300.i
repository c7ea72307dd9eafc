/*
 * SWIG block for SDMPluginGB300::SDMForce, for %include from the reference's
 * python/SDMplugin.i beside its LangevinIntegratorSDM block (that module
 * already imports OpenMM's SWIG headers and std_vector.i).  Plain numbers in
 * OpenMM's internal units (nm, kJ/mol, rad), like the integrator's setters.
 * Not run through SWIG in this repository (SWIG is not installed); the C++
 * interface it wraps is tested in tests/test_openmm_shim.py.
 */
%{
#include "SDMForceGB300.h"
%}

%include "typemaps.i"

namespace SDMPluginGB300 {

class SDMForce : public OpenMM::Force {
public:
    SDMForce(const OpenMM::NonbondedForce& nb, int device = 0);

    void setLambda(double v);
    double getLambda() const;
    void setBiasMethod(int m);
    int getBiasMethod() const;
    void setSoftCoreMethod(int m);
    int getSoftCoreMethod() const;
    void setGamma(double v);
    double getGamma() const;
    void setWBcoeff(double v);
    double getWBcoeff() const;
    void setW0coeff(double v);
    double getW0coeff() const;
    void setLambda1(double v);
    double getLambda1() const;
    void setLambda2(double v);
    double getLambda2() const;
    void setAlpha(double v);
    double getAlpha() const;
    void setU0(double v);
    double getU0() const;
    void setUmax(double v);
    double getUmax() const;
    void setAcore(double v);
    double getAcore() const;
    void setUbcore(double v);
    double getUbcore() const;
    void setNonEquilibrium(int v);
    int getNonEquilibrium() const;
    void setNoneqtmax(double t);
    double getNoneqtmax() const;
    double getNoneqWorkvalue(OpenMM::Context& context);
    void setNoneqWorkvalue(OpenMM::Context& context, double work);
    void setlambda1Slope(double v);
    double getlambda1Slope() const;
    void setlambda2Slope(double v);
    double getlambda2Slope() const;
    void setu0Slope(double v);
    double getu0Slope() const;
    void setw0Slope(double v);
    double getw0Slope() const;
    void setlambda1intercept(double v);
    double getlambda1intercept() const;
    void setlambda2intercept(double v);
    double getlambda2intercept() const;
    void setu0intercept(double v);
    double getu0intercept() const;
    void setw0intercept(double v);
    double getw0intercept() const;
    void setDisplacement(int atom, double dx, double dy, double dz);
    OpenMM::Vec3 getDisplacement(int atom) const;
    int getNumParticles() const;

    void updateParametersInContext(OpenMM::Context& context);
    std::vector<double> getResults(OpenMM::Context& context);
    double getBindE(OpenMM::Context& context);
    double getPotEnergy(OpenMM::Context& context);

    %apply double& OUTPUT { double& u, double& u0, double& u1, double& w, double& dw };
    void getPerturbationEnergy(OpenMM::Context& context, double& u, double& u0, double& u1, double& w, double& dw);
    %clear double& u, double& u0, double& u1, double& w, double& dw;

    bool usesPeriodicBoundaryConditions() const;
};

}
