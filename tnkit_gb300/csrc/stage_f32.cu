// Staging kernels of the tensor-core matvec (sm_103a):
//
//  * cvt_split_kernel: FP64 canonical blocks -> FP32 TF32-split operands in the padded, K-major
//    layout the TMA loads (optionally transposing a block), hi = tf32(x) at dst, lo =
//    tf32(x - hi) at dst + lo_off. 32 x 32 tiles through shared memory keep both the FP64 reads
//    and the FP32 writes coalesced when a block is transposed.
//  * comb_f32_kernel: stage 2 of the mixed matvec (the MPO coefficients) on FP32 data, writing
//    the hi/lo split of its result when the next stage is a split-precision GEMM.
#include "tnk_internal.cuh"

namespace tnk {

// One staged block: source (rows x cols, row stride src_ld) -> destination (cols x rows when
// transposed, row stride dst_ld).
struct CvtTask {
    int64_t src_off, dst_off;
    int32_t rows, cols, src_ld, dst_ld;
    int32_t transpose, pad;
};
static_assert(sizeof(CvtTask) == 40, "CvtTask layout");

struct CvtItem {
    int32_t task, r0, c0, pad;
};

namespace {

__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// grid: one CTA per 32 x 32 source tile (items); 32 x 8 threads
__global__ void __launch_bounds__(256)
cvt_split_kernel(const CvtTask* __restrict__ tasks, const CvtItem* __restrict__ items,
                 const double* __restrict__ src, float* __restrict__ dst, int64_t lo_off,
                 int split) {
    __shared__ double tile[32][33];
    pdl_trigger();
    const CvtItem it = items[blockIdx.x];
    const CvtTask t = tasks[it.task];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    pdl_wait();
    // load 32 x 32 source tile (rows r0.., cols c0..), coalesced along columns
    for (int i = ty; i < 32; i += 8) {
        const int r = it.r0 + i, c = it.c0 + tx;
        tile[i][tx] = (r < t.rows && c < t.cols) ? src[t.src_off + (int64_t)r * t.src_ld + c]
                                                 : 0.0;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        int r, c;
        double x;
        if (t.transpose) {      // destination row = source column
            r = it.c0 + i;      // dst row
            c = it.r0 + tx;     // dst col
            if (r >= t.cols || c >= t.rows) continue;
            x = tile[tx][i];
        } else {
            r = it.r0 + i;
            c = it.c0 + tx;
            if (r >= t.rows || c >= t.cols) continue;
            x = tile[i][tx];
        }
        const int64_t o = t.dst_off + (int64_t)r * t.dst_ld + c;
        const float h = split ? tf32_hi((float)x) : (float)x;
        dst[o] = h;
        if (split) dst[lo_off + o] = tf32_hi((float)(x - (double)h));
    }
}

constexpr int NT = 256;
constexpr int TERMS_SMEM = 64;
constexpr int YSPLIT = 4;       // CTAs per item (gridDim.y): each takes every YSPLIT-th pass

// grid: (items, YSPLIT); each pass covers EPT * NT consecutive elements of the item's row range.
// An element's sum runs over the task's terms in order whatever the split, so the result does not
// depend on the grid; the loads of TB terms are issued together before their FMAs, so a pass waits
// for about one load latency per TB terms rather than one per term.
__global__ void __launch_bounds__(NT)
comb_f32_kernel(const tnk_comb_task* __restrict__ tasks, const tnk_comb_term* __restrict__ terms,
                const tnk_comb_item* __restrict__ items, const float* __restrict__ src,
                float* __restrict__ dst, int64_t lo_off, int split) {
    constexpr int EPT = 4;                      // elements per thread per pass
    constexpr int TB = 4;                       // terms whose loads are in flight together
    __shared__ tnk_comb_term st[TERMS_SMEM];
    pdl_trigger();
    const tnk_comb_item item = items[blockIdx.x];
    const tnk_comb_task t = tasks[item.task];
    const int cols = t.cols;
    const int64_t nel = (int64_t)(item.row1 - item.row0) * cols;
    const bool nel32 = nel <= 0x7fffffff;       // element indices fit 32-bit division
    const int nterm = t.term_end - t.term_begin;
    const bool resident = nterm <= TERMS_SMEM;  // terms staged once for every pass
    if (resident && (int)threadIdx.x < nterm) st[threadIdx.x] = terms[t.term_begin + threadIdx.x];
    __syncthreads();
    pdl_wait();     // src is the previous kernel's output
    for (int64_t e0 = (int64_t)blockIdx.y * EPT * NT; e0 < nel;
         e0 += (int64_t)gridDim.y * EPT * NT) {
        int r[EPT], c[EPT];
        bool live[EPT];
        float acc[EPT];
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
            const int64_t e = e0 + u * NT + (int)threadIdx.x;
            live[u] = e < nel;
            int rr = 0, cc = 0;
            if (live[u]) {
                if (nel32) {
                    const int e32 = (int)e;
                    rr = e32 / cols;
                    cc = e32 - rr * cols;
                } else {
                    rr = (int)(e / cols);
                    cc = (int)(e - (int64_t)rr * cols);
                }
            }
            r[u] = item.row0 + rr;
            c[u] = cc;
            acc[u] = 0.f;
        }
        for (int t0 = 0; t0 < nterm; t0 += TERMS_SMEM) {
            const int nt = min(TERMS_SMEM, nterm - t0);
            if (!resident) {
                __syncthreads();
                if ((int)threadIdx.x < nt) st[threadIdx.x] = terms[t.term_begin + t0 + threadIdx.x];
                __syncthreads();
            }
            for (int q0 = 0; q0 < nt; q0 += TB) {
                float x[TB][EPT];
#pragma unroll
                for (int j = 0; j < TB; ++j) {
                    const bool on = q0 + j < nt;
                    const tnk_comb_term tq = st[on ? q0 + j : q0];
#pragma unroll
                    for (int u = 0; u < EPT; ++u)
                        x[j][u] = (on && live[u]) ? src[tq.src_off + (int64_t)r[u] * tq.src_ld +
                                                        (int64_t)c[u] * tq.src_cs]
                                                  : 0.f;
                }
#pragma unroll
                for (int j = 0; j < TB; ++j) {
                    if (q0 + j < nt) {
                        const float coef = (float)st[q0 + j].coef;
#pragma unroll
                        for (int u = 0; u < EPT; ++u) acc[u] = fmaf(coef, x[j][u], acc[u]);
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
            if (!live[u]) continue;
            const int64_t o = t.dst_off + (int64_t)r[u] * t.dst_ld + (int64_t)c[u] * t.dst_cs;
            const float h = split ? tf32_hi(acc[u]) : acc[u];
            dst[o] = h;
            if (split) dst[lo_off + o] = tf32_hi(acc[u] - h);
        }
    }
}

}  // namespace

int launch_cvt_split(const CvtTask* tasks, const CvtItem* items, int64_t n_items,
                     const double* src, float* dst, int64_t lo_off, int split,
                     cudaStream_t stream) {
    if (n_items < 0 || n_items > 0x7fffffff) {
        set_error("convert: bad item count");
        return TNK_ERR_ARG;
    }
    if (n_items == 0) return TNK_OK;
    if (!tasks || !items || !src || !dst) {
        set_error("convert: null argument");
        return TNK_ERR_ARG;
    }
    cvt_split_kernel<<<(unsigned)n_items, 256, 0, stream>>>(tasks, items, src, dst, lo_off,
                                                            split);
    return check_launch("cvt_split_kernel");
}

int launch_comb_f32(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                    const tnk_comb_item* items, int64_t n_items, const float* src, float* dst,
                    int64_t lo_off, int split, cudaStream_t stream, bool pdl) {
    if (n_items < 0 || n_items > 0x7fffffff) {
        set_error("combine f32: bad item count");
        return TNK_ERR_ARG;
    }
    if (n_items == 0) return TNK_OK;
    if (!tasks || !items || !src || !dst) {
        set_error("combine f32: null argument");
        return TNK_ERR_ARG;
    }
    return launch_k("comb_f32_kernel", comb_f32_kernel, dim3((unsigned)n_items, YSPLIT), dim3(NT),
                    0, stream, pdl, tasks, terms, items, src, dst, lo_off, split);
}

}  // namespace tnk
