// xss_selftest.cu -- self test of the device-side bounded waits.
//
// Every wait in the library's kernels (the decoupled look-back spin, the
// mbarrier wait for a bulk copy) gives up after a spin limit, raises
// XSS_DEVERR_TIMEOUT in the error word and lets the kernel finish.  This entry
// point runs those same waits against conditions that never become true -- a
// look-back predecessor that never publishes, an mbarrier phase nothing
// arrives on -- with a short limit, so a test can show that a stuck wait ends
// with XSS_ETIMEOUT and that the context stays usable afterwards.  Nothing
// here faults or traps.
//
// It also checks the property the radix pass's ranking rests on (RANK 2 in
// xss_onesweep.cuh): shared-memory atomicAdd results of the lanes of one warp
// instruction that meet at one address come back in lane order.
#include "xss_onesweep.cuh"

namespace xss {

__global__ void __launch_bounds__(RADIX / 4) selftest_lookback_kernel(const uint32_t *status,
                                                                      unsigned *err, uint32_t limit)
{
    // tile 1 of a two-tile pass whose tile 0 never publishes (all words
    // zero); four digits per thread as in the pass kernels' vector walk
    uint32_t excl[4];
    lookback_excl<8, 4>(status, 1u, 0u, threadIdx.x * 4, err, excl, limit);
}

__global__ void __launch_bounds__(32) selftest_mbar_kernel(unsigned *err, uint32_t limit)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // no arrival and no copy is ever issued: phase 0 never completes
    (void)mbar_wait_bounded(&bar, 0u, err, limit);
}

// Lane order of same-address shared atomics: every warp counts hashed digits
// (all 256 digits, 16, 4 or a single one; all lanes or a random subset) into
// its own counters and compares each result with the first peer's result
// plus the number of peers in lower lanes.  All accesses are in bounds.
__device__ __forceinline__ uint32_t selftest_hash(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

__global__ void __launch_bounds__(1024) selftest_rank_order_kernel(uint32_t seed, int iters,
                                                                   unsigned long long *viol)
{
    __shared__ uint32_t cnt[32][RADIX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 32 * RADIX; i += 1024) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const uint32_t masks[4] = {RADIX - 1, 15u, 3u, 0u};
    const uint32_t lt = (1u << lane) - 1u;
    unsigned long long bad = 0;
    for (int it = 0; it < iters; ++it) {
        const uint32_t h = selftest_hash(seed ^ (blockIdx.x * 7919u) ^ (warp * 104729u) ^
                                         (it * 2654435761u) ^ (lane * 40503u));
        const uint32_t d = h & masks[it & 3];
        const bool active = (it & 4) == 0 || (selftest_hash(h) & 3u) != 0u;
        const uint32_t am = __ballot_sync(0xffffffffu, active);
        if (active) {
            const uint32_t r = atomicAdd(&cnt[warp][d], 1u);
            const uint32_t peers = __match_any_sync(am, d);
            const uint32_t r0 = __shfl_sync(am, r, __ffs(peers) - 1);
            if (r != r0 + (uint32_t)__popc(peers & lt)) ++bad;
        }
        __syncwarp();
    }
    if (bad) atomicAdd(viol, bad);
}

}  // namespace xss

using namespace xss;

extern "C" int xss_gpu_selftest_rank_order(unsigned long long *violations, xss_stream_t stream)
{
    if (violations == nullptr) return XSS_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    void *ws = nullptr;
    int rc = cached_workspace(s, 4096, &ws);
    if (rc) return rc;
    unsigned long long *viol = static_cast<unsigned long long *>(ws);
    XSS_CUDA_TRY(cudaMemsetAsync(viol, 0, sizeof(*viol), s));
    selftest_rank_order_kernel<<<num_sms(), 1024, 0, s>>>(0x5eed1234u, 2048, viol);
    XSS_CUDA_TRY(cudaGetLastError());
    unsigned long long h = 0;
    XSS_CUDA_TRY(cudaMemcpyAsync(&h, viol, sizeof(h), cudaMemcpyDeviceToHost, s));
    XSS_CUDA_TRY(cudaStreamSynchronize(s));
    *violations = h;
    return XSS_OK;
}

extern "C" int xss_gpu_selftest_bounded_wait(int which, unsigned spin_limit, xss_stream_t stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    void *ws = nullptr;
    int rc = cached_workspace(s, 4096, &ws);
    if (rc) return rc;
    unsigned *err = static_cast<unsigned *>(ws);
    uint32_t *status = reinterpret_cast<uint32_t *>(static_cast<char *>(ws) + 256);
    XSS_CUDA_TRY(cudaMemsetAsync(ws, 0, 256 + 2 * RADIX * sizeof(uint32_t), s));
    if (which == 0) selftest_lookback_kernel<<<1, RADIX / 4, 0, s>>>(status, err, spin_limit);
    else if (which == 1) selftest_mbar_kernel<<<1, 32, 0, s>>>(err, spin_limit);
    else return XSS_EINVAL;
    XSS_CUDA_TRY(cudaGetLastError());
    unsigned h = 0;
    XSS_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(h), cudaMemcpyDeviceToHost, s));
    XSS_CUDA_TRY(cudaStreamSynchronize(s));
    return (h & XSS_DEVERR_TIMEOUT) ? XSS_ETIMEOUT : XSS_OK;
}
