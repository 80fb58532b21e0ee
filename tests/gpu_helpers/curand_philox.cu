// Test helper: the first n 32-bit outputs of cuRAND's Philox4_32_10 generator
// for (seed, subsequence), through cuRAND's public device API.  Used only to
// cross-check the library's and the oracle's Philox-4x32-10 against an
// independent implementation.
#include <cuda_runtime.h>
#include <curand_kernel.h>

__global__ void curand_philox_words(unsigned long long seed, unsigned long long subseq, int n,
                                    unsigned *out)
{
    curandStatePhilox4_32_10_t st;
    curand_init(seed, subseq, 0, &st);
    for (int i = 0; i < n; ++i)
        out[i] = curand(&st);
}

extern "C" int curand_words(unsigned long long seed, unsigned long long subseq, int n, unsigned *host)
{
    unsigned *d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned) * n) != cudaSuccess)
        return -1;
    curand_philox_words<<<1, 1>>>(seed, subseq, n, d);
    cudaError_t e = cudaMemcpy(host, d, sizeof(unsigned) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : -2;
}
