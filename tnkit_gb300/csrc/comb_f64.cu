// Stage 2 of the block contractions: strided linear combinations of sub-matrices (sm_103a).
//
// dst(r, c) = sum_t coef_t * src_t(r, c). The MPO tensors enter the matvec and the environment
// updates here as scalar coefficients, and the same kernel performs block gathers (fuse, split,
// canonical reorder) as one-term combinations. HBM-bound: each CTA owns a chunk of rows of one
// task, stages that task's terms in shared memory and streams the sources once per term.
#include "tnk_internal.cuh"

namespace tnk {
namespace {

constexpr int NT = 256;
constexpr int TERMS_SMEM = 64;

__global__ void __launch_bounds__(NT)
comb_f64_kernel(const tnk_comb_task* __restrict__ tasks, const tnk_comb_term* __restrict__ terms,
                const tnk_comb_item* __restrict__ items, const double* __restrict__ src,
                double* __restrict__ dst) {
    __shared__ tnk_comb_term st[TERMS_SMEM];
    const tnk_comb_item item = items[blockIdx.x];
    const tnk_comb_task t = tasks[item.task];
    const int cols = t.cols;
    const int64_t nel = (int64_t)(item.row1 - item.row0) * cols;
    const int nterm = t.term_end - t.term_begin;
    if (nterm == 0) {
        for (int64_t e = threadIdx.x; e < nel; e += NT) {
            const int r = item.row0 + (int)(e / cols), c = (int)(e % cols);
            dst[t.dst_off + (int64_t)r * t.dst_ld + (int64_t)c * t.dst_cs] = 0.0;
        }
        return;
    }
    for (int t0 = 0; t0 < nterm; t0 += TERMS_SMEM) {
        const int nt = min(TERMS_SMEM, nterm - t0);
        __syncthreads();
        if (threadIdx.x < nt) st[threadIdx.x] = terms[t.term_begin + t0 + threadIdx.x];
        __syncthreads();
        for (int64_t e = threadIdx.x; e < nel; e += NT) {
            const int r = item.row0 + (int)(e / cols), c = (int)(e % cols);
            double acc = 0.0;
            for (int q = 0; q < nt; ++q) {
                const tnk_comb_term& u = st[q];
                acc = fma(u.coef, src[u.src_off + (int64_t)r * u.src_ld + (int64_t)c * u.src_cs],
                          acc);
            }
            double* p = dst + t.dst_off + (int64_t)r * t.dst_ld + (int64_t)c * t.dst_cs;
            *p = (t0 == 0) ? acc : *p + acc;
        }
    }
}

}  // namespace

int launch_comb_f64(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                    const tnk_comb_item* items, int64_t n_items, const double* src,
                    double* dst, cudaStream_t stream) {
    if (n_items < 0 || n_items > 0x7fffffff) {
        set_error("combine: bad item count %lld", (long long)n_items);
        return TNK_ERR_ARG;
    }
    if (n_items == 0) return TNK_OK;
    if (!tasks || !items || !dst || !src) {
        set_error("combine: null table or buffer pointer");
        return TNK_ERR_ARG;
    }
    comb_f64_kernel<<<(unsigned)n_items, NT, 0, stream>>>(tasks, terms, items, src, dst);
    return check_launch("comb_f64_kernel");
}

}  // namespace tnk
