// selftest.cu -- device self-tests exposed through the C ABI:
//   * stencil_selftest_div: the division-by-coefficient fast path (div_coeff,
//     Markstein's method) against the compiler's IEEE division, for every one
//     of the 2^32 float bit patterns;
//   * stencil_selftest_wait: a bounded mbarrier wait that nothing completes
//     gives up after the given limit and sets the device status word, leaving
//     the context usable (the error path of every bounded wait in the kernels).
#include "host.hpp"

namespace st {

template <int C>
__global__ void k_selftest_div(unsigned long long *bad, unsigned *first) {
    unsigned long long local = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += stride) {
        const float x = __uint_as_float((unsigned)i);
        const float a = div_coeff<C>(x);
        const float b = __fdiv_rn(x, (float)C);
        const bool same = __float_as_uint(a) == __float_as_uint(b) || (isnan(a) && isnan(b));
        if (!same) {
            ++local;
            atomicMin(first, (unsigned)i);
        }
    }
    if (local) atomicAdd(bad, local);
}

__global__ void k_selftest_wait(unsigned long long limit_ns, int *result) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);  // one arrival expected; none ever comes
        fence_mbar_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
    if (threadIdx.x == 0) *result = ok ? 1 : 0;
}

namespace {

template <int C>
int run_div(unsigned long long *d_bad, unsigned *d_first) {
    k_selftest_div<C><<<8 * num_sms(), 256>>>(d_bad, d_first);
    return cuda_fail(cudaGetLastError(), "selftest_div launch");
}

}  // namespace

}  // namespace st

using namespace st;

extern "C" int stencil_selftest_div(int coeff, unsigned long long *mismatches,
                                    unsigned *first_mismatch) {
    if (!mismatches) return fail(STENCIL_EINVAL, "null pointer");
    unsigned long long *d_bad = nullptr;
    unsigned *d_first = nullptr;
    ST_CUDA(cudaMalloc(&d_bad, sizeof(unsigned long long) + sizeof(unsigned)));
    d_first = reinterpret_cast<unsigned *>(d_bad + 1);
    int rc = cuda_fail(cudaMemset(d_bad, 0, sizeof(unsigned long long)), "memset");
    const unsigned ff = 0xffffffffu;
    if (!rc) rc = cuda_fail(cudaMemcpy(d_first, &ff, sizeof ff, cudaMemcpyHostToDevice), "memcpy");
    if (!rc) {
        switch (coeff) {
            case 4: rc = run_div<4>(d_bad, d_first); break;
            case 6: rc = run_div<6>(d_bad, d_first); break;
            case 8: rc = run_div<8>(d_bad, d_first); break;
            case 12: rc = run_div<12>(d_bad, d_first); break;
            case 16: rc = run_div<16>(d_bad, d_first); break;
            case 18: rc = run_div<18>(d_bad, d_first); break;
            case 24: rc = run_div<24>(d_bad, d_first); break;
            case 32: rc = run_div<32>(d_bad, d_first); break;
            case 36: rc = run_div<36>(d_bad, d_first); break;
            case 48: rc = run_div<48>(d_bad, d_first); break;
            case 64: rc = run_div<64>(d_bad, d_first); break;
            case 96: rc = run_div<96>(d_bad, d_first); break;
            default: rc = fail(STENCIL_EINVAL, "no kernel uses coefficient %d", coeff);
        }
    }
    if (!rc) rc = cuda_fail(cudaMemcpy(mismatches, d_bad, sizeof *mismatches, cudaMemcpyDeviceToHost), "memcpy");
    if (!rc && first_mismatch)
        rc = cuda_fail(cudaMemcpy(first_mismatch, d_first, sizeof *first_mismatch, cudaMemcpyDeviceToHost), "memcpy");
    cudaFree(d_bad);
    return rc;
}

extern "C" int stencil_selftest_wait(int limit_ms, int *completed, int *status) {
    if (!completed || !status || limit_ms < 1 || limit_ms > 2000)
        return fail(STENCIL_EINVAL, "limit_ms must be in [1, 2000]");
    int *d = nullptr;
    ST_CUDA(cudaMalloc(&d, sizeof(int)));
    k_selftest_wait<<<1, 32>>>((unsigned long long)limit_ms * 1000000ull, d);
    int rc = cuda_fail(cudaGetLastError(), "selftest_wait launch");
    if (!rc) rc = cuda_fail(cudaMemcpy(completed, d, sizeof(int), cudaMemcpyDeviceToHost), "memcpy");
    cudaFree(d);
    if (!rc) rc = stencil_device_status(status);
    return rc;
}
