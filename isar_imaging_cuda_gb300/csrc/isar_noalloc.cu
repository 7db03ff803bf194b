// HRRP centring + 512-cell cut without any memory allocation.
//
// isar_center_cut_noalloc runs the same kernels as isar_stage_center_cut
// (average range profile, HRRPCenter decisions, cutRangeProfile), but takes no
// context: its scratch lives in one file-scope __device__ array, so neither a
// call nor its one-time set-up allocates device or host memory.
//
// Scratch (per device, 65,792 bytes, sized for range_num <= kMaxN = 8192):
//   [0, kMaxN)                 floats  column sums of |y| over the first 256 rows
//   [kMaxN, 2 kMaxN)           floats  average range profile
//   word 2 kMaxN               unsigned max |y| (float bits), atomicMax target
//   words 2 kMaxN + 32 .. +47  ints     centring decisions
// Only the max word has to start at zero; every call zeroes it on the stream
// before its first use.  Everything else is fully written before it is read.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <mutex>

#include "../../include/isar_gb300.h"
#include "isar_common.cuh"
#include "isar_kernels.h"

namespace {

using isar::kMaxN;
using isar::kRangeCut;

constexpr int kHmaxWord = 2 * kMaxN;
constexpr int kDecWord = 2 * kMaxN + 32;   // 128 bytes after the max word
constexpr int kScratchWords = 2 * kMaxN + 64;

static __device__ __align__(256) float g_center_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::atomic<float*> g_scratch_addr[kMaxDevices];
std::mutex g_setup_mu;

int cuda_fail(const char* what, cudaError_t e)
{
    char buf[256];
    snprintf(buf, sizeof(buf), "%s failed: %s", what, cudaGetErrorString(e));
    return isar::record_error(ISAR_ECUDA, buf);
}

// Once per device, with that device current: the scratch's device address and
// k_center's shared-memory limit.  Neither call allocates.
int scratch_for_current_device(float** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail("cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return isar::record_error(ISAR_EINVAL, "device ordinal out of range");
    float* p = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (p) {
        *out = p;
        return ISAR_OK;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    p = g_scratch_addr[dev].load(std::memory_order_relaxed);
    if (!p) {
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_center_scratch);
        if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress(g_center_scratch)", e);
        e = isar::center_prepare_current_device();
        if (e != cudaSuccess) return cuda_fail("cudaFuncSetAttribute(k_center)", e);
        g_scratch_addr[dev].store(p, std::memory_order_release);
    }
    *out = p;
    return ISAR_OK;
}

}  // namespace

ISAR_API int isar_center_cut_noalloc(const float* d_profiles, int echo_num, int range_num, float* d_cut,
                                     void* stream)
{
    const bool setup_only = !d_profiles && !d_cut && echo_num == 0 && range_num == 0;
    if (!setup_only) {
        if (!d_profiles || !d_cut) return isar::record_error(ISAR_EINVAL, "null argument");
        if (range_num > kMaxN) {
            char buf[160];
            snprintf(buf, sizeof(buf), "range_num %d exceeds the static scratch of isar_center_cut_noalloc (%d cells)",
                     range_num, kMaxN);
            return isar::record_error(ISAR_EINVAL, buf);
        }
        if (range_num < kRangeCut || (range_num & (range_num - 1)) != 0)
            return isar::record_error(ISAR_EINVAL, "range_num must be a power of two in [512, 8192]");
        // the pulse counts every other entry point accepts (isar_create)
        if (echo_num < 128 || echo_num > isar::kMaxM || (echo_num & (echo_num - 1)) != 0)
            return isar::record_error(ISAR_EINVAL, "echo_num must be a power of two in [128, 1024]");
    }
    float* s = nullptr;
    const int rc = scratch_for_current_device(&s);
    if (rc != ISAR_OK || setup_only) return rc;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float2* y = reinterpret_cast<const float2*>(d_profiles);
    unsigned* hmax = reinterpret_cast<unsigned*>(s + kHmaxWord);
    int* dec = reinterpret_cast<int*>(s + kDecWord);
    cudaError_t e = isar::arp_from_y(y, echo_num, range_num, s, hmax, s + kMaxN, st);
    if (e != cudaSuccess) return cuda_fail("average range profile", e);
    e = isar::center_cut(s + kMaxN, y, echo_num, range_num, dec, reinterpret_cast<float2*>(d_cut), st);
    if (e != cudaSuccess) return cuda_fail("centring and cut", e);
    return ISAR_OK;
}
