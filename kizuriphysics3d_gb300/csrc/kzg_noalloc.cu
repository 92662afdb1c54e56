// kzg_noalloc.cu - kzg_state_hash_noalloc: PhysicsWorld::ComputeStateHash
// (src/World/PhysicsWorld.cpp:1145-1175) over body state held in the caller's own device buffers,
// without allocating anything, on the host or the device.
//
// The per-body words (packed BodyID, then the 13 state floats scaled by 1e5 and truncated to
// i64) are written in parallel into a fixed file-scope scratch array; one thread then folds them
// with FNV-1a in slot order and leaves the 64-bit result in the same array, and 8 bytes are
// copied back.  The scratch address is looked up once per device with cudaGetSymbolAddress.
//
// Scratch layout (unsigned long long words):
//   [0, 14 n)            words of the current call; every word read is written first by the same
//                        call, so nothing has to start at zero
//   [kResult]            the folded hash, written by the fold before the copy back
// Calls on one device share this scratch: two calls in flight at once on the same device (two
// streams, two host threads) race on it and both results are undefined.  Serialise them.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/kzg.h"

namespace {

constexpr uint32_t kMaxBodies = KZG_NOALLOC_HASH_MAX_BODIES;
constexpr uint32_t kWordsPerBody = 14;
constexpr size_t kResult = size_t(kWordsPerBody) * kMaxBodies;
constexpr int kMaxDevices = 64;

// 14 x 16384 x 8 B = 1.75 MiB of words plus one 256-byte line for the result.
static __device__ __align__(256) unsigned long long g_hash_scratch[kResult + 32];

std::mutex g_setup_mutex;
unsigned long long* g_scratch_ptr[kMaxDevices] = {};

__global__ void k_hash_words_state13(const float* __restrict__ state, const uint32_t* __restrict__ ids, uint32_t n,
                                     unsigned long long* __restrict__ words) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* s = state + 13ull * i;
    unsigned long long* w = words + size_t(kWordsPerBody) * i;
    w[0] = ids[i];
    for (int k = 0; k < 13; ++k) w[1 + k] = (unsigned long long)(long long)(s[k] * 100000.0f);
}

// FNV-1a is a strict left fold; one thread runs it, reading 8 words ahead.
__global__ void k_fnv1a_fold(const unsigned long long* __restrict__ words, size_t count, unsigned long long* result) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    unsigned long long h = 1469598103934665603ull;
    size_t i = 0;
    for (; i + 8 <= count; i += 8) {
        unsigned long long v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = words[i + k];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            h ^= v[k];
            h *= 1099511628211ull;
        }
    }
    for (; i < count; ++i) {
        h ^= words[i];
        h *= 1099511628211ull;
    }
    *result = h;
}

kzg_status fail(const char** error, const char* msg, kzg_status code) {
    if (error) *error = msg;
    return code;
}

// Memory this device's kernels may read: device memory of this very device, or managed memory.
// Device memory of another GPU is refused (without peer access a kernel reading it would fault).
bool device_readable(const void* p, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" kzg_status kzg_state_hash_noalloc(const float* state, const uint32_t* packed_ids, uint32_t n, void* stream,
                                             uint64_t* out, const char** error) {
    if (error) *error = nullptr;
    if (!out) return fail(error, "kzg_state_hash_noalloc: out is NULL", KZG_ERR_INVALID);
    if (n > kMaxBodies)
        return fail(error, "kzg_state_hash_noalloc: more than KZG_NOALLOC_HASH_MAX_BODIES (16384) bodies",
                    KZG_ERR_CAPACITY);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(error, "kzg_state_hash_noalloc: no usable CUDA device", KZG_ERR_CUDA);
    }
    unsigned long long* scratch;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {  // once per device
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_hash_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return fail(error, "kzg_state_hash_noalloc: cudaGetSymbolAddress of the scratch array failed",
                            KZG_ERR_CUDA);
            }
            g_scratch_ptr[dev] = static_cast<unsigned long long*>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    if (n && (!state || !packed_ids || !device_readable(state, dev) || !device_readable(packed_ids, dev)))
        return fail(error, "kzg_state_hash_noalloc: state and packed_ids must be device pointers of the current device",
                    KZG_ERR_INVALID);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Launched through cudaLaunchKernel so that each launch's own status is checked, not an error an
    // earlier call left on this thread.
    cudaError_t e = cudaSuccess;
    if (n) {
        uint32_t nn = n;
        unsigned long long* w = scratch;
        void* args[] = {(void*)&state, (void*)&packed_ids, (void*)&nn, (void*)&w};
        e = cudaLaunchKernel((const void*)k_hash_words_state13, dim3((n + 255) / 256), dim3(256), args, 0, s);
    }
    if (e == cudaSuccess) {
        const unsigned long long* w = scratch;
        size_t count = size_t(kWordsPerBody) * n;
        unsigned long long* res = scratch + kResult;
        void* args[] = {(void*)&w, (void*)&count, (void*)&res};
        e = cudaLaunchKernel((const void*)k_fnv1a_fold, dim3(1), dim3(32), args, 0, s);
    }
    if (e != cudaSuccess) return fail(error, "kzg_state_hash_noalloc: a kernel launch failed", KZG_ERR_CUDA);
    unsigned long long h = 0;
    if (cudaMemcpyAsync(&h, scratch + kResult, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(error, "kzg_state_hash_noalloc: the result copy failed", KZG_ERR_CUDA);
    *out = h;
    return KZG_OK;
}
