// FP64 FMA throughput probe: the denominator of the FP64 roofline that
// bench.py reports next to the HBM one (the diffusion sweeps are bound by the
// FP64 pipe, whose rate is not in the machine's measured peaks).  Eight
// independent FMA chains per thread; the launch shape is the caller's.
#include "dgb_common.cuh"
#include "dgb_internal.h"

namespace dgb {
__global__ void k_fp64_fma(double *out, int iters, int active_lanes)
{
    if ((int)(threadIdx.x & 31) >= active_lanes)
        return;
    double v[8];
#pragma unroll
    for (int c = 0; c < 8; c++)
        v[c] = threadIdx.x * 1e-3 + c;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++)
            v[c] = fma(v[c], 1.0000001, 1e-9);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++)
        s += v[c];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_rcp(const double *x, double *out, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = rcp_full(x[i]);
}
} // namespace dgb

extern "C" int dgb_probe_fp64_fma(double *out, int blocks, int threads, int iters,
                                  int active_lanes, void *stream)
{
    if (!out || blocks < 1 || threads < 32 || threads > 1024 || iters < 1 || active_lanes < 1 ||
        active_lanes > 32)
        return DGB_ERR_ARG;
    dgb::k_fp64_fma<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters, active_lanes);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

extern "C" int dgb_probe_rcp(const double *x, double *out, int n, void *stream)
{
    if (!x || !out || n < 0)
        return DGB_ERR_ARG;
    if (n == 0)
        return DGB_OK;
    dgb::k_rcp<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(x, out, n);
    return cudaGetLastError() == cudaSuccess ? DGB_OK : DGB_ERR_CUDA;
}

namespace dgb {
int preload_probe() { return preload(k_fp64_fma) + preload(k_rcp); }
} // namespace dgb
