// Declarations shared by the translation units of libdadi_gb300.so.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/dadi_gb300.h"

#define DGB_B2_MAXG 8

namespace dgb {
int k2_smem_fits(int Lmax, bool gam_smem, bool delj, size_t *bytes);
int k2_integrate_table(double *phi, int L, const double *xx, const double *table, int nsteps,
                       int frozen_mask, int nomut_mask, int use_delj, void *ws, size_t ws_bytes,
                       cudaStream_t st);
size_t k2_table_ws_bytes(int L);
size_t k2_batch_ws_bytes(int Lmax, long nwork);
} // namespace dgb
