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

}  // namespace xss

using namespace xss;

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
