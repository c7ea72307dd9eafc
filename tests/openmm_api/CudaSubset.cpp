// Bodies of the CUDA-platform subset declared in openmm/cuda/CudaSubset.h
// (test stand-ins, not OpenMM's implementation).  Particles are stored in a
// shuffled order (a fixed permutation) so that the plugin's gather through
// the atom index and its scatter into the fixed-point buffer are exercised.
#include "openmm/cuda/CudaSubset.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <numeric>

namespace OpenMM {

namespace {
void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw OpenMMException(std::string("CUDA stand-in: ") + what + ": " + cudaGetErrorString(e));
}
}  // namespace

CudaArray::~CudaArray() {
    if (pointer) cudaFree((void*)pointer);
}

void CudaArray::initialize(size_t n, int esize, const std::string&) {
    void* p = nullptr;
    ck(cudaMalloc(&p, n * esize), "cudaMalloc");
    ck(cudaMemset(p, 0, n * esize), "cudaMemset");
    pointer = (CUdeviceptr)p;
    size = n;
    elementSize = esize;
}

void CudaArray::upload(const void* data) { ck(cudaMemcpy((void*)pointer, data, size * elementSize, cudaMemcpyHostToDevice), "upload"); }
void CudaArray::download(void* data) const { ck(cudaMemcpy(data, (void*)pointer, size * elementSize, cudaMemcpyDeviceToHost), "download"); }

CudaContext::CudaContext(const System& system, int device, const std::string& prec)
    : deviceIndex(device), numAtoms(system.getNumParticles()), precision(prec) {
    paddedNumAtoms = 32 * ((numAtoms + 31) / 32);
    // a fixed shuffle: stored slot k holds particle atomIndex[k]
    atomIndex.resize(numAtoms);
    std::iota(atomIndex.begin(), atomIndex.end(), 0);
    uint64_t st = 0x9e3779b97f4a7c15ull;
    for (int i = numAtoms - 1; i > 0; --i) {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        std::swap(atomIndex[i], atomIndex[(int)(st % (uint64_t)(i + 1))]);
    }
}

CudaContext::~CudaContext() {
    if (stream) cudaStreamDestroy((cudaStream_t)stream);
}

void CudaContext::allocate() {
    if (posq.isInitialized()) return;
    ck(cudaSetDevice(deviceIndex), "cudaSetDevice");
    cudaStream_t s = nullptr;
    ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    stream = (CUstream)s;
    const int esize = getUseDoublePrecision() ? 32 : 16;
    posq.initialize(paddedNumAtoms, esize, "posq");
    if (getUseMixedPrecision()) posqCorrection.initialize(paddedNumAtoms, 16, "posqCorrection");
    atomIndexDevice.initialize(paddedNumAtoms, 4, "atomIndex");
    std::vector<int> idx(paddedNumAtoms);
    for (int k = 0; k < paddedNumAtoms; ++k) idx[k] = k < numAtoms ? atomIndex[k] : k;
    atomIndexDevice.upload(idx.data());
    longForceBuffer.initialize(3 * (size_t)paddedNumAtoms, 8, "longForceBuffer");
}

// OpenMM's mixed precision: posq = (float) x, posqCorrection = (float) (x - posq)
void CudaContext::uploadPositions(const std::vector<Vec3>& positions) {
    allocate();
    if (getUseDoublePrecision()) {
        std::vector<double> h(4 * (size_t)paddedNumAtoms, 0.0);
        for (int k = 0; k < numAtoms; ++k)
            for (int c = 0; c < 3; ++c) h[4 * k + c] = positions[atomIndex[k]][c];
        posq.upload(h.data());
        return;
    }
    std::vector<float> h(4 * (size_t)paddedNumAtoms, 0.0f), hc(4 * (size_t)paddedNumAtoms, 0.0f);
    for (int k = 0; k < numAtoms; ++k)
        for (int c = 0; c < 3; ++c) {
            const double x = positions[atomIndex[k]][c];
            h[4 * k + c] = (float)x;
            hc[4 * k + c] = (float)(x - (double)h[4 * k + c]);
        }
    posq.upload(h.data());
    if (getUseMixedPrecision()) posqCorrection.upload(hc.data());
}

void CudaContext::clearForces() {
    allocate();
    ck(cudaMemsetAsync((void*)longForceBuffer.getDevicePointer(), 0, 3 * (size_t)paddedNumAtoms * 8, (cudaStream_t)stream),
       "clear forces");
}

void CudaContext::addForcesTo(std::vector<Vec3>& forces) {
    ck(cudaStreamSynchronize((cudaStream_t)stream), "synchronise");
    std::vector<long long> h(3 * (size_t)paddedNumAtoms);
    longForceBuffer.download(h.data());
    const double scale = 1.0 / 4294967296.0;
    for (int k = 0; k < numAtoms; ++k)
        for (int c = 0; c < 3; ++c) forces[atomIndex[k]][c] += (double)h[(size_t)c * paddedNumAtoms + k] * scale;
}

const std::string& CudaPlatform::getName() const {
    static const std::string name = "CUDA";
    return name;
}

void CudaPlatform::contextCreated(ContextImpl& context) const {
    PlatformData* data = new PlatformData();
    data->contexts.push_back(new CudaContext(context.getSystem(), deviceIndex, precision));
    context.setPlatformData(data);
}

void CudaPlatform::contextDestroyed(ContextImpl& context) const {
    PlatformData* data = static_cast<PlatformData*>(context.getPlatformData());
    for (CudaContext* c : data->contexts) delete c;
    delete data;
}

void CudaPlatform::positionsChanged(ContextImpl& context) const {
    std::vector<Vec3> p;
    context.getPositions(p);
    static_cast<PlatformData*>(context.getPlatformData())->contexts[0]->uploadPositions(p);
}

void CudaPlatform::beginForces(ContextImpl& context) const {
    static_cast<PlatformData*>(context.getPlatformData())->contexts[0]->clearForces();
}

void CudaPlatform::endForces(ContextImpl& context) const {
    static_cast<PlatformData*>(context.getPlatformData())->contexts[0]->addForcesTo(context.getForceAccumulator());
}

}  // namespace OpenMM
