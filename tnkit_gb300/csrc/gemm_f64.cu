// Grouped, segmented-K FP64 GEMM over charge blocks (sm_103a).
//
// One CTA computes one 64 x 64 output tile of one task: C = sum_seg coef * A_seg * B_seg, the
// segments being the charge sectors (and MPO channel sectors) summed into that output block.
// Operands are strided views into the caller's flat block buffers: A(i,k) = a[i*a_rs + k*a_cs],
// B(k,j) = b[k*b_rs + j*b_cs]. The loaders pick a coalesced thread mapping from the strides
// (K- or M/N-contiguous), stage 64 x 16 / 16 x 64 tiles through double-buffered shared memory
// with a register prefetch of the next tile, and each thread accumulates a 4 x 4 sub-tile with
// FP64 FMAs. FP64 on GB300 is a scarce unit, so the kernel is bound by FP64 issue, not by HBM:
// the whole operand traffic of a tile is a few bytes per FMA from L2.
#include "tnk_internal.cuh"

namespace tnk {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;
constexpr int PADA = BM + 1, PADB = BN + 1;
// the DMMA tile's row stride: 68 doubles put the four k rows of a fragment load 8 banks apart,
// so the 16 lanes of each half-warp read 16 distinct bank pairs
constexpr int PADD = BM + 4;

struct SegView {
    const double* a;
    const double* b;
    int64_t a_rs, a_cs, b_rs, b_cs;
    int k;
    double coef;
};

__device__ __forceinline__ void load_a(const SegView& s, int m0, int M, int k0, int tid,
                                       double (&ra)[4]) {
    const bool kc = (s.a_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int mm = kc ? (idx >> 4) : (idx & (BM - 1));
        const int kk = kc ? (idx & (BK - 1)) : (idx >> 6);
        const int m = m0 + mm, k = k0 + kk;
        ra[r] = (m < M && k < s.k) ? s.a[(int64_t)m * s.a_rs + (int64_t)k * s.a_cs] * s.coef : 0.0;
    }
}

template <int PAD = PADA>
__device__ __forceinline__ void store_a(const SegView& s, int tid, const double (&ra)[4],
                                        double* As) {
    const bool kc = (s.a_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int mm = kc ? (idx >> 4) : (idx & (BM - 1));
        const int kk = kc ? (idx & (BK - 1)) : (idx >> 6);
        As[kk * PAD + mm] = ra[r];
    }
}

__device__ __forceinline__ void load_b(const SegView& s, int n0, int N, int k0, int tid,
                                       double (&rb)[4]) {
    const bool nc = (s.b_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int nn = nc ? (idx & (BN - 1)) : (idx >> 4);
        const int kk = nc ? (idx >> 6) : (idx & (BK - 1));
        const int n = n0 + nn, k = k0 + kk;
        rb[r] = (n < N && k < s.k) ? s.b[(int64_t)k * s.b_rs + (int64_t)n * s.b_cs] : 0.0;
    }
}

template <int PAD = PADB>
__device__ __forceinline__ void store_b(const SegView& s, int tid, const double (&rb)[4],
                                        double* Bs) {
    const bool nc = (s.b_cs == 1);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int idx = tid + r * NT;
        const int nn = nc ? (idx & (BN - 1)) : (idx >> 4);
        const int kk = nc ? (idx >> 6) : (idx & (BK - 1));
        Bs[kk * PAD + nn] = rb[r];
    }
}

__global__ void __launch_bounds__(NT, 2)
gemm_f64_kernel(const tnk_gemm_task* __restrict__ tasks, const tnk_gemm_seg* __restrict__ segs,
                const tnk_gemm_tile* __restrict__ tiles, Slots slots, double* __restrict__ C) {
    __shared__ double As[2][BK * PADA];
    __shared__ double Bs[2][BK * PADB];
    const tnk_gemm_tile tile = tiles[blockIdx.x];
    const tnk_gemm_task task = tasks[tile.task];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int M = task.m, N = task.n, m0 = tile.m0, n0 = tile.n0;

    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    int cur = 0;
    for (int si = task.seg_begin; si < task.seg_end; ++si) {
        const tnk_gemm_seg g = segs[si];
        SegView s;
        s.a = slots.p[g.a_buf] + g.a_off;
        s.b = slots.p[g.b_buf] + g.b_off;
        s.a_rs = g.a_rs; s.a_cs = g.a_cs; s.b_rs = g.b_rs; s.b_cs = g.b_cs;
        s.k = g.k; s.coef = g.coef;
        if (s.k <= 0) continue;
        double ra[4], rb[4];
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
            const double* as = As[cur];
            const double* bs = Bs[cur];
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                double a[4], b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = as[kk * PADA + ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = bs[kk * PADB + tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
            }
            if (more) {
                store_a(s, tid, ra, As[cur ^ 1]);
                store_b(s, tid, rb, Bs[cur ^ 1]);
            }
            __syncthreads();
            cur ^= 1;
        }
    }

    const bool accumulate = (task.flags & 1) != 0;
    // flags bit 2: output column stride 2 (the real or imaginary half of interleaved complex);
    // bit 4: a split-K partial product, written to the workspace (slot 3) instead of C
    const int64_t ccs = (task.flags & 4) ? 2 : 1;
    double* c = ((task.flags & 16) ? const_cast<double*>(slots.p[3]) : C) + task.c_off;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n >= N) continue;
            double* p = c + (int64_t)m * task.ldc + (int64_t)n * ccs;
            *p = accumulate ? *p + acc[i][j] : acc[i][j];
        }
    }
}


// The same tile on the FP64 tensor path: mma.sync m8n8k4 (DMMA) instead of per-thread FMAs.
// Eight warps as a 2 x 4 grid of 32 x 16 warp tiles; per K step of 4 each warp issues 4 x 2
// MMAs from 4 A fragments (a = A[lane/4][lane%4] of an 8 x 4 slice) and 2 B fragments
// (b = B[lane%4][lane/4] of a 4 x 8 slice), accumulating c = C[lane/4][2 (lane%4) + {0, 1}] of
// each 8 x 8 tile in registers. Loaders, shared-memory tiles and the epilogue's flags are the
// FMA kernel's; only the inner product differs (one instruction per 512 flops instead of 2).
__device__ __forceinline__ void dmma_8x8x4(double& c0, double& c1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                 : "+d"(c0), "+d"(c1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(NT, 2)
gemm_f64_dmma_kernel(const tnk_gemm_task* __restrict__ tasks,
                     const tnk_gemm_seg* __restrict__ segs, const tnk_gemm_tile* __restrict__ tiles,
                     Slots slots, double* __restrict__ C) {
    __shared__ double As[2][BK * PADD];
    __shared__ double Bs[2][BK * PADD];
    const tnk_gemm_tile tile = tiles[blockIdx.x];
    const tnk_gemm_task task = tasks[tile.task];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
    const int g = lane >> 2, q = lane & 3;
    const int M = task.m, N = task.n, m0 = tile.m0, n0 = tile.n0;

    double acc[4][2][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    int cur = 0;
    for (int si = task.seg_begin; si < task.seg_end; ++si) {
        const tnk_gemm_seg sg = segs[si];
        SegView s;
        s.a = slots.p[sg.a_buf] + sg.a_off;
        s.b = slots.p[sg.b_buf] + sg.b_off;
        s.a_rs = sg.a_rs; s.a_cs = sg.a_cs; s.b_rs = sg.b_rs; s.b_cs = sg.b_cs;
        s.k = sg.k; s.coef = sg.coef;
        if (s.k <= 0) continue;
        double ra[4], rb[4];
        load_a(s, m0, M, 0, tid, ra);
        load_b(s, n0, N, 0, tid, rb);
        store_a<PADD>(s, tid, ra, As[cur]);
        store_b<PADD>(s, tid, rb, Bs[cur]);
        __syncthreads();
        for (int k0 = 0; k0 < s.k; k0 += BK) {
            const bool more = k0 + BK < s.k;
            if (more) {
                load_a(s, m0, M, k0 + BK, tid, ra);
                load_b(s, n0, N, k0 + BK, tid, rb);
            }
            const double* as = As[cur];
            const double* bs = Bs[cur];
#pragma unroll
            for (int kk = 0; kk < BK; kk += 4) {
                double a[4], b[2];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = as[(kk + q) * PADD + wm + 8 * i + g];
#pragma unroll
                for (int j = 0; j < 2; ++j) b[j] = bs[(kk + q) * PADD + wn + 8 * j + g];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 2; ++j) dmma_8x8x4(acc[i][j][0], acc[i][j][1], a[i], b[j]);
            }
            if (more) {
                store_a<PADD>(s, tid, ra, As[cur ^ 1]);
                store_b<PADD>(s, tid, rb, Bs[cur ^ 1]);
            }
            __syncthreads();
            cur ^= 1;
        }
    }

    const bool accumulate = (task.flags & 1) != 0;
    const int64_t ccs = (task.flags & 4) ? 2 : 1;
    double* c = ((task.flags & 16) ? const_cast<double*>(slots.p[3]) : C) + task.c_off;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + wm + 8 * i + g;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int n = n0 + wn + 8 * j + 2 * q + h;
                if (n >= N) continue;
                double* p = c + (int64_t)m * task.ldc + (int64_t)n * ccs;
                *p = accumulate ? *p + acc[i][j][h] : acc[i][j][h];
            }
        }
    }
}

int g_gemm_f64_variant = 0;     // 0: FP64 FMA tile, 1: DMMA tile (tnk_gemm_f64_variant)

}  // namespace

// Selects the inner product of every FP64 grouped GEMM launched afterwards (process-wide).
extern "C" int tnk_gemm_f64_variant(int32_t variant) {
    const int prev = g_gemm_f64_variant;
    if (variant == 0 || variant == 1) g_gemm_f64_variant = variant;
    return prev;
}

int launch_gemm_f64(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                    const tnk_gemm_tile* tiles, int64_t n_tiles, Slots slots, double* C,
                    cudaStream_t stream) {
    if (n_tiles < 0 || n_tiles > 0x7fffffff) {
        set_error("grouped gemm: bad tile count %lld", (long long)n_tiles);
        return TNK_ERR_ARG;
    }
    if (n_tiles == 0) return TNK_OK;
    if (!tasks || !segs || !tiles || !C) {
        set_error("grouped gemm: null table or output pointer");
        return TNK_ERR_ARG;
    }
    if (g_gemm_f64_variant == 1) {
        gemm_f64_dmma_kernel<<<(unsigned)n_tiles, NT, 0, stream>>>(tasks, segs, tiles, slots, C);
        return check_launch("gemm_f64_dmma_kernel");
    }
    gemm_f64_kernel<<<(unsigned)n_tiles, NT, 0, stream>>>(tasks, segs, tiles, slots, C);
    return check_launch("gemm_f64_kernel");
}

}  // namespace tnk
