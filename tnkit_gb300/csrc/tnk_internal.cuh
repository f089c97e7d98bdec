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

// Programmatic dependent launch. A kernel launched by launch_k with pdl = true may be scheduled
// while its predecessor in the stream still runs -- once every CTA of the predecessor has called
// pdl_trigger or exited -- and must call pdl_wait before it touches memory the predecessor (or
// anything before it) writes or reads; pdl_wait returns when the predecessor has completed and
// its writes are visible. For a kernel launched plainly both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch k<<<grid, block, smem, stream>>>(args...), with programmatic stream serialisation
// when pdl.
template <typename... KArgs, typename... Args>
inline int launch_k(const char* what, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                    cudaStream_t stream, bool pdl, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k, args...);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        set_error("%s: %s", what, cudaGetErrorString(e));
        return TNK_ERR_CUDA;
    }
    return check_launch(what);
}

}  // namespace tnk
