/*
 * Declarations of the part of OpenMM's CUDA platform (OpenMM 8) that the
 * plugin's CalcSDMForce kernel uses: CudaPlatform and its PlatformData,
 * CudaContext's position, atom-index and 64-bit force arrays, its precision
 * flags, device and stream, and CudaArray's device pointer.  Class and
 * method names and signatures are OpenMM's; the bodies (CudaSubset.cpp) are
 * test stand-ins: one context, device arrays from the CUDA runtime, particles
 * stored in a fixed shuffled order, forces read back from the fixed-point
 * buffer after every evaluation.  Not OpenMM's implementation.
 */
#ifndef OPENMM_CUDA_SUBSET_H
#define OPENMM_CUDA_SUBSET_H

#include "../ApiSubset.h"

#include <cuda.h>

#include <string>
#include <vector>

namespace OpenMM {

class CudaArray {
public:
    CudaArray() {}
    ~CudaArray();
    CudaArray(const CudaArray&) = delete;
    CudaArray& operator=(const CudaArray&) = delete;
    void initialize(size_t size, int elementSize, const std::string& name);
    bool isInitialized() const { return pointer != 0; }
    size_t getSize() const { return size; }
    int getElementSize() const { return elementSize; }
    CUdeviceptr& getDevicePointer() { return pointer; }
    void upload(const void* data);
    void download(void* data) const;

private:
    CUdeviceptr pointer = 0;
    size_t size = 0;
    int elementSize = 0;
};

class CudaContext {
public:
    /* precision: "single", "mixed" or "double" (as OpenMM's Precision property) */
    CudaContext(const System& system, int deviceIndex, const std::string& precision);
    ~CudaContext();
    int getDeviceIndex() const { return deviceIndex; }
    int getNumAtoms() const { return numAtoms; }
    int getPaddedNumAtoms() const { return paddedNumAtoms; }
    bool getUseDoublePrecision() const { return precision == "double"; }
    bool getUseMixedPrecision() const { return precision == "mixed"; }
    CudaArray& getPosq() { return posq; }
    CudaArray& getPosqCorrection() { return posqCorrection; }
    CudaArray& getAtomIndexArray() { return atomIndexDevice; }
    const std::vector<int>& getAtomIndex() const { return atomIndex; }
    CudaArray& getLongForceBuffer() { return longForceBuffer; }
    CUstream getCurrentStream() { return stream; }
    // stand-in internals (not OpenMM API)
    void uploadPositions(const std::vector<Vec3>& positions);
    void clearForces();
    void addForcesTo(std::vector<Vec3>& forces);

private:
    void allocate();
    int deviceIndex, numAtoms, paddedNumAtoms;
    std::string precision;
    std::vector<int> atomIndex;
    CudaArray posq, posqCorrection, atomIndexDevice, longForceBuffer;
    CUstream stream = nullptr;
};

class CudaPlatform : public Platform {
public:
    struct PlatformData {
        std::vector<CudaContext*> contexts;
    };
    /* precision of the contexts this platform creates (stand-in setting) */
    explicit CudaPlatform(const std::string& precision = "mixed", int deviceIndex = 0)
        : precision(precision), deviceIndex(deviceIndex) {}
    const std::string& getName() const override;
    void contextCreated(ContextImpl& context) const override;
    void contextDestroyed(ContextImpl& context) const override;
    void positionsChanged(ContextImpl& context) const override;
    void beginForces(ContextImpl& context) const override;
    void endForces(ContextImpl& context) const override;

private:
    std::string precision;
    int deviceIndex;
};

}  // namespace OpenMM

#endif
