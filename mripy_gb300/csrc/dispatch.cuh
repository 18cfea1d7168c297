// Template dispatch over (dimension, taps per dimension, coils per block).
#pragma once
#include <mutex>
#include <unordered_map>

#include "grid_kernels.cuh"

namespace gbn {

// compile-time tap counts; any other W uses the generic (runtime W) instantiation
#define GBN_DISPATCH_W(W, ...)                                  \
    do {                                                        \
        if ((W) == 12) { constexpr int WT = 12; __VA_ARGS__; }  \
        else if ((W) == 10) { constexpr int WT = 10; __VA_ARGS__; } \
        else { constexpr int WT = 0; __VA_ARGS__; }             \
    } while (0)

#define GBN_DISPATCH_CG(CGV, ...)                               \
    do {                                                        \
        if ((CGV) == 8) { constexpr int CG = 8; __VA_ARGS__; }  \
        else if ((CGV) == 4) { constexpr int CG = 4; __VA_ARGS__; } \
        else if ((CGV) == 2) { constexpr int CG = 2; __VA_ARGS__; } \
        else { constexpr int CG = 1; __VA_ARGS__; }             \
    } while (0)

#define GBN_DISPATCH_D(DV, ...)                                 \
    do {                                                        \
        if ((DV) == 3) { constexpr int D = 3; __VA_ARGS__; }    \
        else if ((DV) == 2) { constexpr int D = 2; __VA_ARGS__; } \
        else { constexpr int D = 1; __VA_ARGS__; }              \
    } while (0)

// Raise a kernel's dynamic shared-memory limit once per (kernel, size); later launches
// (including those recorded during graph capture) skip the attribute call.
template <typename K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    static std::mutex mu;
    static std::unordered_map<const void *, size_t> done;
    std::lock_guard<std::mutex> lock(mu);
    auto it = done.find((const void *)kernel);
    if (it != done.end() && it->second >= bytes) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) done[(const void *)kernel] = bytes;
    return e;
}

}  // namespace gbn
