// Host-only stand-ins for the two CUDA runtime calls that the reference's
// CPU instantiation GPMA<CPU> still makes: it moves host scalars with
// cudaMemcpy(HostToHost) (gpma.cuh:860,868 via utils.cuh:99-102) and calls
// cudaDeviceSynchronize. Without a GPU driver the real runtime refuses both,
// so the reference oracle binary links these definitions ahead of the shared
// runtime. Only the host-to-host kind is legal here.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime_api.h>

extern "C" cudaError_t cudaMemcpy(void *dst, const void *src, size_t count, cudaMemcpyKind kind) {
    if (kind != cudaMemcpyHostToHost && kind != cudaMemcpyDefault) {
        std::fprintf(stderr, "h2h_shim: cudaMemcpy kind %d is not host-to-host\n", (int)kind);
        std::abort();
    }
    std::memmove(dst, src, count);
    return cudaSuccess;
}

extern "C" cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
