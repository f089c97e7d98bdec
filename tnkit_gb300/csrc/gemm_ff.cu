// Grouped segmented-K GEMM in float-float ("double-FP32") arithmetic on the FP32 CUDA cores.
//
// GB300 runs FP32 FMAs ~70x faster than FP64 ones. Operands are unevaluated pairs hi + lo of
// floats (hi = fl(x), lo = fl(x - hi): 48 significant bits), split once from FP64 by
// ff_split_kernel into buffers with the FP64 layout (a float2 is as wide as a double, so every
// offset of the plan tables stays valid). Each multiply-add of a tile uses error-free
// transformations: the exact product error of hi*hi from an FMA, the cross terms hi*lo + lo*hi,
// and Knuth's two-sum into the accumulator pair; the lo*lo term (2^-48 relative) is dropped and
// the pair is renormalised once per 16-wide K tile. No FP64 instruction runs in the inner loop.
// Stage-1 outputs stay float-float (task flags bit 3), stage 2 combines float-float blocks with
// the MPO coefficients, stage 3 writes FP64. Accurate to ~1e-13 relative on the H_eff
// contractions.
//
// The kernels read the same task, segment and tile tables as the FP64 ones (64 x 64 tiles,
// strided operands, segmented K, output column stride 2 for complex halves).
#include "tnk_internal.cuh"

namespace tnk {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;
constexpr int PADA = BM + 1, PADB = BN + 1;

struct SegView {
    const float2* a;
    const float2* b;
    int64_t a_rs, a_cs, b_rs, b_cs;
    int k;
    float neg;            // the segment coefficient, +1 or -1 (checked on the host)
};

__device__ __forceinline__ float2 scale_pm(float2 x, float s) {
    return make_float2(x.x * s, x.y * s);   // exact for s = +-1
}

__device__ __forceinline__ void load_a(const SegView& s, int m0, int M, int k0, int tid,
                                       float2 (&ra)[4]) {
    const bool kc = (s.a_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int mm = kc ? (idx >> 4) : (idx & (BM - 1));
        const int kk = kc ? (idx & (BK - 1)) : (idx >> 6);
        const int m = m0 + mm, k = k0 + kk;
        ra[r] = (m < M && k < s.k)
                    ? scale_pm(s.a[(int64_t)m * s.a_rs + (int64_t)k * s.a_cs], s.neg)
                    : make_float2(0.f, 0.f);
    }
}

__device__ __forceinline__ void store_a(const SegView& s, int tid, const float2 (&ra)[4],
                                        float2* As) {
    const bool kc = (s.a_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int mm = kc ? (idx >> 4) : (idx & (BM - 1));
        const int kk = kc ? (idx & (BK - 1)) : (idx >> 6);
        As[kk * PADA + mm] = ra[r];
    }
}

__device__ __forceinline__ void load_b(const SegView& s, int n0, int N, int k0, int tid,
                                       float2 (&rb)[4]) {
    const bool nc = (s.b_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int nn = nc ? (idx & (BN - 1)) : (idx >> 4);
        const int kk = nc ? (idx >> 6) : (idx & (BK - 1));
        const int n = n0 + nn, k = k0 + kk;
        rb[r] = (n < N && k < s.k) ? s.b[(int64_t)k * s.b_rs + (int64_t)n * s.b_cs]
                                   : make_float2(0.f, 0.f);
    }
}

__device__ __forceinline__ void store_b(const SegView& s, int tid, const float2 (&rb)[4],
                                        float2* Bs) {
    const bool nc = (s.b_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int nn = nc ? (idx & (BN - 1)) : (idx >> 4);
        const int kk = nc ? (idx >> 6) : (idx & (BK - 1));
        Bs[kk * PADB + nn] = rb[r];
    }
}

// c += a * b in float-float (lo*lo dropped, no renormalisation). The _rn intrinsics are never
// contracted into FMAs, which would break the error-free transformations.
__device__ __forceinline__ void ff_mac(float2& c, const float2 a, const float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = fmaf(a.x, b.x, -p);                       // exact error of the hi*hi product
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float s = __fadd_rn(c.x, p);                  // two-sum of c.x + p
    const float v = __fsub_rn(s, c.x);
    const float t = __fadd_rn(__fsub_rn(c.x, __fsub_rn(s, v)), __fsub_rn(p, v));
    c.x = s;
    c.y = __fadd_rn(c.y, __fadd_rn(e, t));
}

__device__ __forceinline__ void ff_renorm(float2& c) {
    const float s = __fadd_rn(c.x, c.y);
    c.y = __fsub_rn(c.y, __fsub_rn(s, c.x));
    c.x = s;
}

__global__ void __launch_bounds__(NT, 2)
gemm_ff_kernel(const tnk_gemm_task* __restrict__ tasks, const tnk_gemm_seg* __restrict__ segs,
               const tnk_gemm_tile* __restrict__ tiles, Slots slots, double* __restrict__ C) {
    __shared__ float2 As[2][BK * PADA];
    __shared__ float2 Bs[2][BK * PADB];
    const tnk_gemm_tile tile = tiles[blockIdx.x];
    const tnk_gemm_task task = tasks[tile.task];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int M = task.m, N = task.n, m0 = tile.m0, n0 = tile.n0;

    float2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);

    int cur = 0;
    for (int si = task.seg_begin; si < task.seg_end; ++si) {
        const tnk_gemm_seg g = segs[si];
        SegView s;
        s.a = reinterpret_cast<const float2*>(slots.p[g.a_buf]) + g.a_off;
        s.b = reinterpret_cast<const float2*>(slots.p[g.b_buf]) + g.b_off;
        s.a_rs = g.a_rs; s.a_cs = g.a_cs; s.b_rs = g.b_rs; s.b_cs = g.b_cs;
        s.k = g.k; s.neg = g.coef < 0 ? -1.f : 1.f;
        if (s.k <= 0) continue;
        float2 ra[4], rb[4];
        load_a(s, m0, M, 0, tid, ra);
        load_b(s, n0, N, 0, tid, rb);
        store_a(s, tid, ra, As[cur]);
        store_b(s, tid, rb, Bs[cur]);
        __syncthreads();
        for (int k0 = 0; k0 < s.k; k0 += BK) {
            const bool more = k0 + BK < s.k;
            if (more) {
                load_a(s, m0, M, k0 + BK, tid, ra);
                load_b(s, n0, N, k0 + BK, tid, rb);
            }
            const float2* as = As[cur];
            const float2* bs = Bs[cur];
#pragma unroll 4
            for (int kk = 0; kk < BK; ++kk) {
                float2 a[4], b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = as[kk * PADA + ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = bs[kk * PADB + tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) ff_mac(acc[i][j], a[i], b[j]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) ff_renorm(acc[i][j]);
            if (more) {
                store_a(s, tid, ra, As[cur ^ 1]);
                store_b(s, tid, rb, Bs[cur ^ 1]);
            }
            __syncthreads();
            cur ^= 1;
        }
    }

    // flags bit 2: output column stride 2; bit 3: float-float output (a float2 per element);
    // bit 4: a split-K partial product (FP64), written to the workspace (slot 3) instead of C
    const int64_t ccs = (task.flags & 4) ? 2 : 1;
    const bool ffout = (task.flags & 8) != 0;
    if (task.flags & 16) C = const_cast<double*>(slots.p[3]);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n >= N) continue;
            const int64_t o = task.c_off + (int64_t)m * task.ldc + (int64_t)n * ccs;
            if (ffout)
                reinterpret_cast<float2*>(C)[o] = acc[i][j];
            else
                C[o] = (double)acc[i][j].x + (double)acc[i][j].y;
        }
    }
}

// x (FP64) -> (hi, lo) float pairs, same element offsets
__global__ void __launch_bounds__(256) ff_split_kernel(const double* __restrict__ x,
                                                       float2* __restrict__ y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        const float h = __double2float_rn(v);
        y[i] = make_float2(h, __double2float_rn(v - (double)h));
    }
}

constexpr int TERMS_SMEM = 64;

// Stage 2 in float-float: dst(r, c) = sum_t coef_t * src_t(r, c) on float2 data; the FP64
// coefficients are split into float pairs and applied with an error-free product.
__global__ void __launch_bounds__(256)
comb_ff_kernel(const tnk_comb_task* __restrict__ tasks, const tnk_comb_term* __restrict__ terms,
               const tnk_comb_item* __restrict__ items, const float2* __restrict__ src,
               float2* __restrict__ dst) {
    __shared__ float4 st[TERMS_SMEM];        // (coef hi, coef lo, ld, cs as floats unused)
    __shared__ int64_t so[TERMS_SMEM];
    __shared__ int sl[TERMS_SMEM], sc[TERMS_SMEM];
    const tnk_comb_item item = items[blockIdx.x];
    const tnk_comb_task t = tasks[item.task];
    const int cols = t.cols;
    const int64_t nel = (int64_t)(item.row1 - item.row0) * cols;
    const int nterm = t.term_end - t.term_begin;
    for (int64_t e0 = 0; e0 < nel; e0 += 256) {
        const int64_t e = e0 + threadIdx.x;
        const bool live = e < nel;
        const int r = live ? item.row0 + (int)(e / cols) : 0;
        const int c = live ? (int)(e % cols) : 0;
        float2 acc = make_float2(0.f, 0.f);
        for (int t0 = 0; t0 < nterm; t0 += TERMS_SMEM) {
            const int nt = min(TERMS_SMEM, nterm - t0);
            __syncthreads();
            if (threadIdx.x < nt) {
                const tnk_comb_term u = terms[t.term_begin + t0 + threadIdx.x];
                const float ch = __double2float_rn(u.coef);
                st[threadIdx.x] = make_float4(ch, __double2float_rn(u.coef - (double)ch), 0.f, 0.f);
                so[threadIdx.x] = u.src_off;
                sl[threadIdx.x] = u.src_ld;
                sc[threadIdx.x] = u.src_cs;
            }
            __syncthreads();
            if (live)
                for (int q = 0; q < nt; ++q) {
                    const float2 x = src[so[q] + (int64_t)r * sl[q] + (int64_t)c * sc[q]];
                    ff_mac(acc, make_float2(st[q].x, st[q].y), x);
                }
        }
        if (live) {
            ff_renorm(acc);
            dst[t.dst_off + (int64_t)r * t.dst_ld + (int64_t)c * t.dst_cs] = acc;
        }
    }
}

}  // namespace

int launch_gemm_ff(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                   const tnk_gemm_tile* tiles, int64_t n_tiles, Slots slots, double* C,
                   cudaStream_t stream) {
    if (n_tiles < 0 || n_tiles > 0x7fffffff) {
        set_error("grouped gemm (ff): bad tile count %lld", (long long)n_tiles);
        return TNK_ERR_ARG;
    }
    if (n_tiles == 0) return TNK_OK;
    if (!tasks || !segs || !tiles || !C) {
        set_error("grouped gemm (ff): null table or output pointer");
        return TNK_ERR_ARG;
    }
    gemm_ff_kernel<<<(unsigned)n_tiles, NT, 0, stream>>>(tasks, segs, tiles, slots, C);
    return check_launch("gemm_ff_kernel");
}

int launch_ff_split(const double* x, double* y, int64_t n, cudaStream_t stream) {
    if (!x || !y || n < 0) {
        set_error("ff split: bad argument");
        return TNK_ERR_ARG;
    }
    if (n == 0) return TNK_OK;
    int64_t g = (n + 1023) / 1024;
    g = (g + 151) / 152 * 152;
    if (g > 152 * 16) g = 152 * 16;
    ff_split_kernel<<<(unsigned)g, 256, 0, stream>>>(x, reinterpret_cast<float2*>(y), n);
    return check_launch("ff_split_kernel");
}

int launch_comb_ff(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                   const tnk_comb_item* items, int64_t n_items, const double* src, double* dst,
                   cudaStream_t stream) {
    if (n_items < 0 || n_items > 0x7fffffff) {
        set_error("combine (ff): bad item count");
        return TNK_ERR_ARG;
    }
    if (n_items == 0) return TNK_OK;
    if (!tasks || !items || !src || !dst) {
        set_error("combine (ff): null argument");
        return TNK_ERR_ARG;
    }
    comb_ff_kernel<<<(unsigned)n_items, 256, 0, stream>>>(
        tasks, terms, items, reinterpret_cast<const float2*>(src), reinterpret_cast<float2*>(dst));
    return check_launch("comb_ff_kernel");
}

}  // namespace tnk

extern "C" {

int tnk_ff_split(const double* x, double* y, int64_t n, void* stream) {
    return tnk::launch_ff_split(x, y, n, (cudaStream_t)stream);
}

int tnk_grouped_gemm_ff(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                        const tnk_gemm_tile* tiles, int64_t n_tiles, const double* b0,
                        const double* b1, const double* b2, const double* b3, double* C,
                        void* stream) {
    tnk::Slots s{{b0, b1, b2, b3}};
    return tnk::launch_gemm_ff(tasks, segs, tiles, n_tiles, s, C, (cudaStream_t)stream);
}

int tnk_contract3_ff(const tnk_plan3* p, const double* x0, const double* x1, const double* x2,
                     double* out, double* ws, int64_t ws_elems, void* stream) {
    if (!p) {
        tnk::set_error("plan3 (ff): null plan");
        return TNK_ERR_ARG;
    }
    if (p->ws1_elems < 0 || p->ws2_elems < 0 || ws_elems < p->ws1_elems + p->ws2_elems) {
        tnk::set_error("plan3 (ff): workspace of %lld elements, plan needs %lld",
                       (long long)ws_elems, (long long)(p->ws1_elems + p->ws2_elems));
        return TNK_ERR_SIZE;
    }
    if (!out || (p->ws1_elems + p->ws2_elems > 0 && !ws)) {
        tnk::set_error("plan3 (ff): null output or workspace");
        return TNK_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    tnk::Slots s{{x0, x1, x2, ws}};
    int rc = tnk::launch_gemm_ff(p->t1, p->s1, p->tiles1, p->n_tiles1, s, ws, st);
    if (rc) return rc;
    rc = tnk::launch_comb_ff(p->t2, p->c2, p->items2, p->n_items2, ws, ws, st);
    if (rc) return rc;
    rc = tnk::launch_gemm_ff(p->t3, p->s3, p->tiles3, p->n_tiles3, s, out, st);
    if (rc) return rc;
    return tnk::launch_comb_f64(p->t4, p->c4, p->items4, p->n_items4, ws, out, st);
}

int tnk_apply_two_site_ff(const tnk_plan3* plan, const double* L2, const double* theta,
                          const double* R2, double* out, double* ws, int64_t ws_elems,
                          void* stream) {
    if (!plan || !L2 || !theta || !R2) {
        tnk::set_error("apply_two_site_ff: null plan or operand");
        return TNK_ERR_ARG;
    }
    const int64_t need = plan->ws1_elems + plan->ws2_elems;
    const int64_t n = plan->out_elems;
    if (ws_elems < need + n || n < 0) {
        tnk::set_error("apply_two_site_ff: workspace of %lld elements, needs %lld (plan + theta)",
                       (long long)ws_elems, (long long)(need + n));
        return TNK_ERR_SIZE;
    }
    double* theta2 = ws + need;
    int rc = tnk::launch_ff_split(theta, theta2, n, (cudaStream_t)stream);
    if (rc) return rc;
    return tnk_contract3_ff(plan, L2, theta2, R2, out, ws, need, stream);
}

}  // extern "C"
