// Declarations shared by the translation units of libdadi_gb300.so.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/dadi_gb300.h"

#define DGB_B2_MAXG 8

#include <mutex>

namespace dgb {
// Raise a kernel's dynamic shared-memory limit to the device's opt-in
// maximum, once per device.  The limit is a per-function setting shared by
// every host thread, so lowering it per launch would race with concurrent
// launches of the same kernel from other threads; it is only ever raised.
// Kernels are told apart by address (template instances share a type).
inline int raise_smem_limit_ptr(const void *kernel)
{
    static std::mutex mu;
    static const void *keys[64];
    static unsigned long long done[64];
    static int nkeys = 0;
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return -2;
    std::lock_guard<std::mutex> g(mu);
    int k = 0;
    while (k < nkeys && keys[k] != kernel)
        k++;
    if (k == nkeys) {
        if (nkeys == 64)
            return -2;
        keys[nkeys] = kernel;
        done[nkeys] = 0;
        nkeys++;
    }
    if (done[k] >> dev & 1ull)
        return 0;
    cudaFuncAttributes fa;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess ||
        cudaFuncGetAttributes(&fa, kernel) != cudaSuccess)
        return -2;
    // the dynamic limit may not exceed the opt-in size minus static shared memory
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - (int)fa.sharedSizeBytes) != cudaSuccess) {
        cudaGetLastError();
        return -2;
    }
    done[k] |= 1ull << dev;
    return 0;
}

template <typename Kernel> inline int raise_smem_limit(Kernel kernel)
{
    return raise_smem_limit_ptr((const void *)kernel);
}

// Load a kernel now (1 if it cannot be).  Under lazy module loading a
// kernel is loaded at its first launch, and loading can wait for the device
// to go idle: a first launch on one stream then serialises behind the work
// other streams have in flight.
template <typename Kernel> inline int preload(Kernel kernel)
{
    cudaFuncAttributes fa;
    return cudaFuncGetAttributes(&fa, (const void *)kernel) == cudaSuccess ? 0 : 1;
}

// Each translation unit's kernels (dgb_preload loads them all).
int preload_integrate2d();
int preload_sweepnd();
int preload_probe();
int preload_adjoint2d();
int preload_fsepi();
int preload_adjointnd();
int preload_batchnd();
int preload_cluster2d();
} // namespace dgb

namespace dgb {
int k2_smem_fits(int Lmax, bool gam_smem, bool delj, size_t *bytes);
int k2_integrate_table(double *phi, int L, const double *xx, const double *table, int nsteps,
                       int frozen_mask, int nomut_mask, int use_delj, void *ws, size_t ws_bytes,
                       cudaStream_t st);
size_t k2_table_ws_bytes(int L);
size_t k2_batch_ws_bytes(int Lmax, long nwork);
} // namespace dgb
