// Jaccard edge weights on device buffers, without any allocation by this library.
//
// Who needs this: code that hands the library device buffers it already owns but is not allowed to
// allocate device memory itself — for example a plug-in running inside a host framework that owns
// every device allocation through its own pool, or a caller whose memory budget is fixed up front.
// costal_reweight allocates its scratch with cudaMalloc on first use; this entry point instead uses a
// fixed scratch array compiled into the library (below), so it never calls cudaMalloc, cudaFree or any
// other allocating routine.
//
// The price: the array (NOALLOC_SCRATCH_BYTES, 16 MiB) is reserved on every GPU that loads the
// library's device code, for as long as the process lives, and it is shared by all calls. With CUDA's
// lazy module loading (the default) that reservation is made when the device code is first used on a
// device, which may be this entry point's first call there: on a device without 16 MiB free that call
// fails with COSTAL_ECUDA. A caller with a fixed budget makes one call at start-up. It holds the row-sorted
// copy of the neighbour matrix, so n·k may be at most NOALLOC_MAX_ENTRIES; larger inputs are rejected
// before any device work. Two calls whose work overlaps on the GPU (different streams, or host
// threads) race on the array and corrupt each other's result: serialise them.

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "costal_gb300.h"

namespace costal {
void note_launch();
}
using costal::note_launch;

namespace {

constexpr size_t NOALLOC_HEADER_BYTES = 256;  // first-bad-index flag, cleared at every call
constexpr size_t NOALLOC_MAX_ENTRIES = 4u << 20;  // n·k ≤ 4,194,304 neighbour entries
constexpr size_t NOALLOC_SCRATCH_BYTES = NOALLOC_HEADER_BYTES + NOALLOC_MAX_ENTRIES * sizeof(uint32_t);

// The scratch: a flag word, then the row-sorted neighbour lists (n·k u32). In host code this name
// is only a stand-in for the device copy; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[MAX_DEVICES] = {};

// Sort each row's neighbour ids into the scratch (insertion sort; k is small). An index outside
// [0, n) records its flat position in the flag and is sorted as 0, so every later read stays in range.
__global__ void k_sort_rows_checked(const int32_t* __restrict__ idx, int n, int k, uint32_t* __restrict__ sorted,
                                    unsigned long long* __restrict__ first_bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t* row = sorted + (size_t)i * k;
    for (int t = 0; t < k; ++t) {
        const int32_t raw = idx[(size_t)i * k + t];
        uint32_t v = (uint32_t)raw;
        if (raw < 0 || raw >= n) {
            atomicMin(first_bad, (unsigned long long)i * k + t);
            v = 0;
        }
        int p = t;
        while (p > 0 && row[p - 1] > v) {
            row[p] = row[p - 1];
            --p;
        }
        row[p] = v;
    }
}

// weight.rs:64-93: s = |N(i) ∩ N(j)| by merging two sorted rows, w = s / (2k − s).
__global__ void k_jaccard_checked(const int32_t* __restrict__ idx, const uint32_t* __restrict__ sorted, int n, int k,
                                  double* __restrict__ out) {
    const uint64_t nk = (uint64_t)n * k;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nk; e += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t raw = idx[e];
        const uint32_t j = (raw < 0 || raw >= n) ? 0u : (uint32_t)raw;
        const uint32_t* a = sorted + (e / k) * k;
        const uint32_t* b = sorted + (size_t)j * k;
        int p = 0, q = 0, c = 0;
        while (p < k && q < k) {
            const uint32_t x = a[p], y = b[q];
            p += x <= y;
            q += y <= x;
            c += x == y;
        }
        const double s = (double)c;
        out[e] = __ddiv_rn(s, __dsub_rn(__dmul_rn(2.0, (double)k), s));
    }
}

void put_err(char* err, size_t errlen, const std::string& msg) {
    if (err && errlen) std::snprintf(err, errlen, "%s", msg.c_str());
}

}  // namespace

extern "C" int costal_reweight_jaccard_device_noalloc(const int32_t* d_idx, uint64_t n, uint32_t k, double* d_out,
                                                      void* stream, char* err, size_t errlen) {
    if (n == 0 || k == 0) return COSTAL_OK;
    // Each factor is checked before the product is formed, so n * k cannot wrap around.
    if (n > NOALLOC_MAX_ENTRIES || k > NOALLOC_MAX_ENTRIES || n * (uint64_t)k > NOALLOC_MAX_ENTRIES) {
        put_err(err, errlen,
                "costal_reweight_jaccard_device_noalloc: n*k = " + std::to_string(n) + "*" + std::to_string(k) +
                    " exceeds the fixed scratch of " + std::to_string(NOALLOC_MAX_ENTRIES) +
                    " neighbour entries; use costal_reweight instead");
        return COSTAL_EINVAL;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        put_err(err, errlen, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
        return COSTAL_ECUDA;
    }
    // Set-up, once per device, with that device current: the first call on a device looks up the
    // array's device address (so make that first call before capturing any stream into a graph).
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mu);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) {
                put_err(err, errlen, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
                return COSTAL_ECUDA;
            }
            g_scratch_addr[dev] = p;
        }
        base = g_scratch_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto* first_bad = static_cast<unsigned long long*>(base);
    auto* sorted = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(base) + NOALLOC_HEADER_BYTES);
    // The flag must start "no bad index" (all ones); the sorted rows are fully rewritten every call.
    if ((e = cudaMemsetAsync(first_bad, 0xff, sizeof(unsigned long long), st)) != cudaSuccess) {
        put_err(err, errlen, std::string("cudaMemsetAsync failed: ") + cudaGetErrorString(e));
        return COSTAL_ECUDA;
    }
    k_sort_rows_checked<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(d_idx, (int)n, (int)k, sorted, first_bad); note_launch();
    k_jaccard_checked<<<1024, 256, 0, st>>>(d_idx, sorted, (int)n, (int)k, d_out); note_launch();
    unsigned long long bad = 0;
    int32_t bad_val = 0;
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(&bad, first_bad, sizeof bad, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
        put_err(err, errlen, std::string("Jaccard kernels failed: ") + cudaGetErrorString(e));
        return COSTAL_ECUDA;
    }
    if (bad != ~0ull) {
        if (cudaMemcpy(&bad_val, d_idx + bad, sizeof bad_val, cudaMemcpyDeviceToHost) != cudaSuccess) bad_val = -1;
        put_err(err, errlen, "neighbor index " + std::to_string(bad_val) + " out of range (n=" + std::to_string(n) + ")");
        return COSTAL_EINVAL;
    }
    return COSTAL_OK;
}
