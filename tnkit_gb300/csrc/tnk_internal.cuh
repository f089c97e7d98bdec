// Internal helpers shared by the CUDA sources of libtnkit_gb300 (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/tnkit_gb300.h"

static_assert(sizeof(tnk_gemm_task) == 32, "tnk_gemm_task layout");
static_assert(sizeof(tnk_gemm_seg) == 56, "tnk_gemm_seg layout");
static_assert(sizeof(tnk_gemm_tile) == 16, "tnk_gemm_tile layout");
static_assert(sizeof(tnk_comb_task) == 32, "tnk_comb_task layout");
static_assert(sizeof(tnk_comb_term) == 24, "tnk_comb_term layout");
static_assert(sizeof(tnk_comb_item) == 16, "tnk_comb_item layout");
static_assert(sizeof(tnk_sytrd_sector) == 32, "tnk_sytrd_sector layout");
static_assert(sizeof(tnk_ormtr_item) == 16, "tnk_ormtr_item layout");
static_assert(sizeof(tnk_gebrd_sector) == 64, "tnk_gebrd_sector layout");
static_assert(sizeof(tnk_refl_set) == 48, "tnk_refl_set layout");

namespace tnk {

// The calling thread's last error message (tnk_last_error).
void set_error(const char* fmt, ...);

// Operand base pointers of a grouped GEMM, by slot.
struct Slots {
    const double* p[4];
};

// Launchers (host side, defined in the .cu files). Each returns TNK_OK or a TNK_ERR_* code.
int launch_gemm_f64(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                    const tnk_gemm_tile* tiles, int64_t n_tiles, Slots slots, double* C,
                    cudaStream_t stream);
int launch_gemm_ff(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                   const tnk_gemm_tile* tiles, int64_t n_tiles, Slots slots, double* C,
                   cudaStream_t stream);
int launch_comb_f64(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                    const tnk_comb_item* items, int64_t n_items, const double* src,
                    double* dst, cudaStream_t stream);

// Check the last launch; record a message on failure.
inline int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return TNK_ERR_CUDA;
    }
    return TNK_OK;
}

}  // namespace tnk
