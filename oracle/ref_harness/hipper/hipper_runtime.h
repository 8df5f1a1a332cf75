// Minimal stand-in for the hipper runtime shim (the reference's extern/hipper submodule is empty),
// used only to compile the reference's own kernels for the reference harness.  Each name maps to
// the CUDA runtime call of the same meaning.
#ifndef NEIGHBOR_REF_HARNESS_HIPPER_RUNTIME_H_
#define NEIGHBOR_REF_HARNESS_HIPPER_RUNTIME_H_

#include <cstddef>
#include <utility>

#include <cuda_runtime.h>

#ifndef HIPPER_PLATFORM_NVCC
#define HIPPER_PLATFORM_NVCC
#endif

namespace hipper
{
typedef cudaStream_t stream_t;
typedef cudaError_t error_t;
static const cudaError_t success = cudaSuccess;
typedef cudaFuncAttributes funcAttributes_t;

inline error_t funcGetAttributes(funcAttributes_t* attr, const void* f) { return cudaFuncGetAttributes(attr, f); }
inline error_t mallocManaged(void** ptr, size_t bytes) { return cudaMallocManaged(ptr, bytes); }
inline error_t free(void* ptr) { return cudaFree(ptr); }
inline error_t memsetAsync(void* ptr, int value, size_t bytes, stream_t stream = 0)
    {
    return cudaMemsetAsync(ptr, value, bytes, stream);
    }
inline error_t streamCreate(stream_t* s) { return cudaStreamCreate(s); }
inline error_t streamDestroy(stream_t s) { return cudaStreamDestroy(s); }
inline error_t streamSynchronize(stream_t s) { return cudaStreamSynchronize(s); }
inline error_t deviceSynchronize() { return cudaDeviceSynchronize(); }

// Global thread index for a 1D grid of 1D blocks.
template<int GRID_DIM, int BLOCK_DIM>
__device__ inline unsigned int threadRank();
template<>
__device__ inline unsigned int threadRank<1, 1>()
    {
    return blockIdx.x * blockDim.x + threadIdx.x;
    }

class KernelLauncher
    {
    public:
        KernelLauncher(dim3 grid, dim3 block, stream_t stream = 0) : grid_(grid), block_(block), stream_(stream) {}
        template<class Kernel, class... Args>
        void operator()(Kernel kernel, Args&&... args)
            {
            kernel<<<grid_, block_, 0, stream_>>>(std::forward<Args>(args)...);
            }
    private:
        dim3 grid_;
        dim3 block_;
        stream_t stream_;
    };
} // namespace hipper

#endif
