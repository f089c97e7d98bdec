// Grouped GEMM over charge blocks on the 5th-generation tensor cores (tcgen05, kind::tf32).
//
// One CTA computes one 128 x BN output tile (BN = 128 or 64) of one task, C = sum_seg A_seg *
// B_seg^T, where every operand is a K-major FP32 block staged by the host planner in a
// 16-byte-aligned padded layout. Operand tiles (128 rows x 32 FP32 = one 128-byte swizzle atom)
// arrive by TMA (cp.async.bulk.tensor.2d, SWIZZLE_128B, out-of-bounds rows/columns zero-filled,
// so ragged sector blocks need no masking) into a shared-memory ring of stages_for(BN) slots;
// one elected thread issues tcgen05.mma with the accumulator in TMEM and releases each slot with
// tcgen05.commit; the epilogue moves the accumulator TMEM -> registers (tcgen05.ld 32x32b) ->
// shared memory -> global, as FP32 (the next stage's input) or FP64 (the Lanczos vector). The
// matvec launches it as a programmatic dependent of the kernel before it (griddepcontrol).
//
// PASSES = 3 is the split-precision product A*B ~ Ah*Bh + Ah*Bl + Al*Bh of TF32 "hi" and "lo"
// parts (each operand stored twice: hi = tf32(x), lo = tf32(x - hi)), accurate to ~1e-6
// relative with FP32 accumulation; PASSES = 1 is plain TF32. PASSES = 4 is the same product as
// PASSES = 3 with the operands staged once, as FP32: each ring slot's tiles arrive raw and six
// splitter warps write the hi part in place and the lo part beside it before the MMAs read them
// (half the bytes from L2 per K step, the stages being bound by that traffic). The parts are
// those of the FP32 value: for FP64-sourced operands (theta, L, R) the staged split rounds the
// FP64 residual x - hi instead, so the two forms differ in the last bit of some lo parts
// (~1e-7 of the result); both are ~1e-6 from FP64.
//
// Every mbarrier wait is bounded; on a timeout the CTA records an error code in `err`, skips
// the rest of its work, waits (bounded) for its own issued operations and frees its TMEM.
#include <cuda.h>

#include "tnk_internal.cuh"

namespace tnk {

// Segment of the tensor-core grouped GEMM: operand tensor maps (hi at index 2i, lo at 2i+1).
struct TcSeg {
    int32_t a_map, b_map, k, pad;
};
static_assert(sizeof(TcSeg) == 16, "TcSeg layout");

namespace {

constexpr int BM = 128, BK = 32;
// Depth of the operand ring: three slots of 64 KB for 128-wide tiles; four of 48 KB for 64-wide
// ones, whose long K loops (stage 3: ~27 K steps per tile) otherwise wait on TMA latency that
// three slots do not cover.
__host__ __device__ constexpr int stages_for(int bnt) { return bnt == 64 ? 4 : 3; }
constexpr int NT = 128;
constexpr int NT4 = 256;                    // PASSES = 4: two more roles of warps (splitters)
constexpr int TILE_BYTES = BM * BK * 4;     // 16 KiB: one A tile (and a B tile of 128 rows)
constexpr unsigned WAIT_LIMIT = 1u << 26;   // tries per mbarrier wait (well over a second)

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// Bounded parity wait: true when the phase completed, false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const uint32_t a = smem_u32(bar);
    for (unsigned i = 0; i < WAIT_LIMIT; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Make host-written tensor maps in global memory visible to the tensor-map proxy.
__device__ __forceinline__ void tmap_acquire(const CUtensorMap* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                     reinterpret_cast<uint64_t>(map))
                 : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(const void* p) {
    const uint64_t addr = smem_u32(p);
    uint64_t d = 0;
    d |= (addr & 0x3FFFFull) >> 4;             // start address (16-byte units), bits 0-13
    d |= (uint64_t)0 << 16;                    // leading byte offset: one swizzle atom on K
    d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset between 8-row groups
    d |= (uint64_t)1 << 46;                    // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                    // layout: SWIZZLE_128B
    return d;
}

// Instruction descriptor of kind::tf32: D = F32, A = B = TF32, both K-major, M = 128, N = BNT.
template <int BNT>
__host__ __device__ constexpr uint32_t idesc_tf32() {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BNT >> 3) << 17) |
           ((uint32_t)(BM >> 4) << 24);
}

template <int BNT>
__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc_tf32<BNT>()), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// Bounded parity wait that also gives up when the CTA's abort flag is raised by the other role.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, unsigned parity,
                                                   volatile int* abort_flag) {
    const uint32_t a = smem_u32(bar);
    for (unsigned i = 0; i < WAIT_LIMIT; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 255) == 255 && *abort_flag) return false;
    }
    return false;
}

// One warp's share of an epilogue: `rows` (<= 32) staged rows of NQ * 32 columns at src (row
// stride lds floats, all 32 rows readable) go to C[base + r * ldc + c] for c < cols. Rows go in
// batches of 32 / NQ: a batch's shared-memory loads all issue before its global stores, so the
// warp waits one load latency per batch rather than one per store (the row-at-a-time loop
// spent ~15 k cycles of a 128 x 128 tile's epilogue on that chain, ~5 k batched).
template <int NQ, typename T>
__device__ __forceinline__ void store_rows(T* __restrict__ C, int64_t base, int64_t ldc,
                                           const float* __restrict__ src, int lds, int rows,
                                           int cols, int lane) {
    constexpr int RB = 32 / NQ;
    for (int r0 = 0; r0 < rows; r0 += RB) {
        float x[RB][NQ];
#pragma unroll
        for (int i = 0; i < RB; ++i)
#pragma unroll
            for (int q = 0; q < NQ; ++q) x[i][q] = src[(r0 + i) * lds + q * 32 + lane];
#pragma unroll
        for (int i = 0; i < RB; ++i)
#pragma unroll
            for (int q = 0; q < NQ; ++q)
                if (r0 + i < rows && q * 32 + lane < cols)
                    C[base + (int64_t)(r0 + i) * ldc + q * 32 + lane] = (T)x[i][q];
    }
}

// Warp roles: warp 0 lane 0 streams the operand tiles by TMA into the STAGES-deep ring (waiting
// for the MMA issuer to release a slot before refilling it), warp 1 lane 0 issues the MMAs as
// tiles land and releases each slot with tcgen05.commit, so loads run STAGES - 1 K steps ahead
// of the tensor core without either thread waiting on its own work. After the last MMA all four
// warps move the accumulator out: TMEM -> registers (32 columns per tcgen05.ld) -> a padded
// shared-memory tile (the operand ring, idle by then) -> global memory in batches of rows
// (store_rows), 32 consecutive columns per store instruction. BNT is the tile width (128, or 64 for stages with
// few, long tasks: twice the CTAs at half the work each), with B tiles of BNT rows.
template <int PASSES, int BNT>
__global__ void __launch_bounds__(PASSES == 4 ? NT4 : NT, 1)
gemm_tc_kernel(const tnk_gemm_task* __restrict__ tasks, const TcSeg* __restrict__ segs,
               const tnk_gemm_tile* __restrict__ tiles, const CUtensorMap* __restrict__ maps,
               void* __restrict__ Cout, int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    constexpr int STAGES = stages_for(BNT);
    constexpr int A_BYTES = TILE_BYTES;                 // 128 x 32 FP32
    constexpr int B_BYTES = BNT * BK * 4;               // BNT x 32 FP32 (a multiple of 1 KiB)
    constexpr int PAIR = A_BYTES + B_BYTES;
    constexpr int STAGE_BYTES = (PASSES >= 3) ? 2 * PAIR : PAIR;  // Ah, Bh (, Al, Bl)
    constexpr bool SPLIT = PASSES == 4;                 // hi/lo formed in shared memory
    constexpr int LOAD_BYTES = SPLIT ? PAIR : STAGE_BYTES;
    constexpr int NSPLIT_W = (NT4 - 64) / 32;           // splitter warps 2 .. 7
    constexpr int LDS = BNT + 1;                        // staging row stride (floats)
    static_assert(BM * LDS * 4 <= STAGES * STAGE_BYTES, "staging tile fits the ring");
    static_assert(B_BYTES % 1024 == 0, "B tiles keep the 1 KiB swizzle alignment");
    uint8_t* base = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* stage_mem = base;
    uint64_t* full = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* done = empty + STAGES;
    uint64_t* splitb = done + 1;                        // PASSES = 4: STAGES split barriers
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(splitb + STAGES);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    int* counts = const_cast<int*>(abort_flag) + 1;     // [0] issued loads, [1] consumed

    pdl_trigger();
    const tnk_gemm_tile tile = tiles[blockIdx.x];
    const tnk_gemm_task task = tasks[tile.task];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(BNT)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 32) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
            if (SPLIT) mbar_init(&splitb[s], NSPLIT_W);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        counts[0] = counts[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    pdl_wait();     // the operands (and C's previous readers) belong to the kernels before

    // total K steps over all segments
    int nk = 0;
    for (int s = task.seg_begin; s < task.seg_end; ++s) nk += (segs[s].k + BK - 1) / BK;

    if (threadIdx.x == 0 && nk > 0) {
        // TMA producer: cursor over (segment, k0)
        int ls = task.seg_begin, lk = 0, issued = 0;
        for (int i = 0; i < nk; ++i) {
            const int slot = i % STAGES;
            if (i >= STAGES &&
                !mbar_wait_or_abort(&empty[slot], ((i / STAGES) - 1) & 1, abort_flag)) {
                if (!*abort_flag) atomicExch(err, 2);
                *abort_flag = 1;
                break;
            }
            while (lk >= segs[ls].k) { ++ls; lk = 0; }
            const TcSeg g = segs[ls];
            if (lk == 0) {
                tmap_acquire(&maps[2 * g.a_map]);
                tmap_acquire(&maps[2 * g.b_map]);
                if (PASSES == 3) {
                    tmap_acquire(&maps[2 * g.a_map + 1]);
                    tmap_acquire(&maps[2 * g.b_map + 1]);
                }
            }
            uint8_t* st = stage_mem + slot * STAGE_BYTES;
            mbar_expect_tx(&full[slot], LOAD_BYTES);
            tma_load_2d(st, &maps[2 * g.a_map], &full[slot], lk, tile.m0);
            tma_load_2d(st + A_BYTES, &maps[2 * g.b_map], &full[slot], lk, tile.n0);
            if (PASSES == 3) {
                tma_load_2d(st + PAIR, &maps[2 * g.a_map + 1], &full[slot], lk, tile.m0);
                tma_load_2d(st + PAIR + A_BYTES, &maps[2 * g.b_map + 1], &full[slot], lk,
                            tile.n0);
            }
            lk += BK;
            ++issued;
        }
        counts[0] = issued;
    } else if (SPLIT && threadIdx.x >= 64 && nk > 0) {
        // splitters (warps 2 .. 7): the raw FP32 tiles of a slot -> hi in place, lo beside them
        // (the same swizzled positions), then a proxy fence so the tensor core sees the writes
        const int t = threadIdx.x - 64;
        for (int i = 0; i < nk; ++i) {
            const int slot = i % STAGES;
            bool ok = true;
            if (lane == 0) ok = mbar_wait_or_abort(&full[slot], (i / STAGES) & 1, abort_flag);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) {
                if (lane == 0) {
                    if (!*abort_flag) atomicExch(err, 4);
                    *abort_flag = 1;
                }
                break;
            }
            float4* hi = reinterpret_cast<float4*>(stage_mem + slot * STAGE_BYTES);
            float4* lo = reinterpret_cast<float4*>(stage_mem + slot * STAGE_BYTES + PAIR);
            for (int e = t; e < PAIR / 16; e += NSPLIT_W * 32) {
                const float4 x = hi[e];
                float4 h, l;
                h.x = tf32_rna(x.x); l.x = tf32_rna(x.x - h.x);
                h.y = tf32_rna(x.y); l.y = tf32_rna(x.y - h.y);
                h.z = tf32_rna(x.z); l.z = tf32_rna(x.z - h.z);
                h.w = tf32_rna(x.w); l.w = tf32_rna(x.w - h.w);
                hi[e] = h;
                lo[e] = l;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                 smem_u32(&splitb[slot]))
                             : "memory");
        }
    } else if (threadIdx.x == 32 && nk > 0) {
        // MMA issuer
        int consumed = 0;
        for (int i = 0; i < nk; ++i) {
            const int slot = i % STAGES;
            if (!mbar_wait_or_abort(SPLIT ? &splitb[slot] : &full[slot], (i / STAGES) & 1,
                                    abort_flag)) {
                if (!*abort_flag) atomicExch(err, 1);
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            uint8_t* st = stage_mem + slot * STAGE_BYTES;
#pragma unroll
            for (int kk = 0; kk < BK / 8; ++kk) {
                const uint64_t ah = smem_desc(st + kk * 32);
                const uint64_t bh = smem_desc(st + A_BYTES + kk * 32);
                mma_tf32<BNT>(tmem, ah, bh, (i > 0 || kk > 0) ? 1u : 0u);
                if (PASSES >= 3) {
                    const uint64_t al = smem_desc(st + PAIR + kk * 32);
                    const uint64_t bl = smem_desc(st + PAIR + A_BYTES + kk * 32);
                    mma_tf32<BNT>(tmem, ah, bl, 1u);
                    mma_tf32<BNT>(tmem, al, bh, 1u);
                }
            }
            mma_commit(&empty[slot]);
            consumed = i + 1;
        }
        counts[1] = consumed;
        mma_commit(done);       // arrives once every MMA issued above has completed
    }
    __syncthreads();
    if (threadIdx.x == 0 && *abort_flag) {
        // drain: wait (bounded) for the TMA copies issued and not consumed, so none lands in
        // shared memory after the CTA has moved on or exited
        for (int j = counts[1]; j < counts[0]; ++j)
            mbar_wait(&full[j % STAGES], (j / STAGES) & 1);
    }
    const bool have_acc = nk > 0;
    bool acc_ready = true;
    if (have_acc) acc_ready = mbar_wait(done, 0);
    if (!acc_ready) atomicExch(err, 3);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // CTA-uniform: TMEM loads are .sync.aligned and must be issued by whole warps
    const int bad = __syncthreads_or((*abort_flag != 0) || !acc_ready);

    // epilogue: warp w < 4 owns accumulator rows 32w..32w+31 (its TMEM lane quarter)
    float* stg = reinterpret_cast<float*>(stage_mem);
    const int rloc = warp * 32 + lane;
    const int tile_cols = min(BNT, task.n - tile.n0);   // chunks past the task's width hold 0
    for (int c0 = 0; c0 < BNT && c0 < tile_cols && warp < 4; c0 += 32) {
        uint32_t v[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0u;
        if (have_acc && !bad) {
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                  "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                  "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]),
                  "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
                  "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                  "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) stg[rloc * LDS + c0 + j] = __uint_as_float(v[j]);
    }
    __syncwarp();
    if (!bad && warp < 4) {
        const bool f64 = (task.flags & 2) != 0;
        const int rows = min(32, task.m - (tile.m0 + warp * 32));
        const int64_t base = task.c_off + (int64_t)(tile.m0 + warp * 32) * task.ldc + tile.n0;
        const float* src = stg + warp * 32 * LDS;
        if (f64)
            store_rows<BNT / 32>(reinterpret_cast<double*>(Cout), base, task.ldc, src, LDS, rows,
                                 tile_cols, lane);
        else
            store_rows<BNT / 32>(reinterpret_cast<float*>(Cout), base, task.ldc, src, LDS, rows,
                                 tile_cols, lane);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(BNT)
                     : "memory");
    }
}

// Persistent form of the same GEMM for stages with more tiles than SMs: one CTA per SM walks
// the tiles blockIdx.x, blockIdx.x + gridDim.x, ... with the operand ring running on across
// tile boundaries and two TMEM accumulators, so the epilogue of one tile overlaps the MMAs of
// the next. Six warps: warp 0 lane 0 the TMA producer, warp 1 lane 0 the MMA issuer, warps 2-5
// the epilogue (warp w reads TMEM lane quarter w % 4, i.e. rows 32 (w % 4) .. + 31 of the
// tile, through its own padded 32 x 33 staging tile). Barriers: the ring's full / empty pair
// per slot; acc_full[b] (the issuer's commit after a tile's last MMA into accumulator b) and
// acc_empty[b] (one arrival per epilogue warp once it has read accumulator b). Every wait is
// bounded and also ends when any role has raised the abort flag; a CTA that aborts records a
// code in `err`, drains its own TMA copies, waits (bounded) for its MMAs and frees its TMEM.
constexpr int NT_P = 192;

template <int PASSES, int BNT>
__global__ void __launch_bounds__(NT_P, 1)
gemm_tc_persistent_kernel(const tnk_gemm_task* __restrict__ tasks,
                          const TcSeg* __restrict__ segs, const tnk_gemm_tile* __restrict__ tiles,
                          int n_tiles, const CUtensorMap* __restrict__ maps,
                          void* __restrict__ Cout, int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    constexpr int STAGES = stages_for(BNT);
    constexpr int A_BYTES = TILE_BYTES;
    constexpr int B_BYTES = BNT * BK * 4;
    constexpr int PAIR = A_BYTES + B_BYTES;
    constexpr int STAGE_BYTES = (PASSES == 3) ? 2 * PAIR : PAIR;
    constexpr int LDW = 33;                               // per-warp staging row stride
    uint8_t* base = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* ring = base;
    float* stg_all = reinterpret_cast<float*>(base + STAGES * STAGE_BYTES);
    uint64_t* full = reinterpret_cast<uint64_t*>(stg_all + 4 * 32 * LDW);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* done = acc_empty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    int* counts = const_cast<int*>(abort_flag) + 1;       // [0] issued loads, [1] consumed

    pdl_trigger();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(2 * BNT)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 32) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        counts[0] = counts[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    pdl_wait();     // the operands (and C's previous readers) belong to the kernels before

    auto ksteps = [&](const tnk_gemm_task& task) {
        int nk = 0;
        for (int s = task.seg_begin; s < task.seg_end; ++s) nk += (segs[s].k + BK - 1) / BK;
        return nk;
    };

    if (threadIdx.x == 0) {
        // TMA producer over every K step of every tile of this CTA, one ring
        int g = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
            const tnk_gemm_tile tile = tiles[t];
            const tnk_gemm_task task = tasks[tile.task];
            int ls = task.seg_begin, lk = 0;
            const int nk = ksteps(task);
            for (int i = 0; i < nk; ++i, ++g) {
                const int slot = g % STAGES;
                if (g >= STAGES &&
                    !mbar_wait_or_abort(&empty[slot], ((g / STAGES) - 1) & 1, abort_flag)) {
                    if (!*abort_flag) atomicExch(err, 12);
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                while (lk >= segs[ls].k) { ++ls; lk = 0; }
                const TcSeg sg = segs[ls];
                if (lk == 0) {
                    tmap_acquire(&maps[2 * sg.a_map]);
                    tmap_acquire(&maps[2 * sg.b_map]);
                    if (PASSES == 3) {
                        tmap_acquire(&maps[2 * sg.a_map + 1]);
                        tmap_acquire(&maps[2 * sg.b_map + 1]);
                    }
                }
                uint8_t* st = ring + slot * STAGE_BYTES;
                mbar_expect_tx(&full[slot], STAGE_BYTES);
                tma_load_2d(st, &maps[2 * sg.a_map], &full[slot], lk, tile.m0);
                tma_load_2d(st + A_BYTES, &maps[2 * sg.b_map], &full[slot], lk, tile.n0);
                if (PASSES == 3) {
                    tma_load_2d(st + PAIR, &maps[2 * sg.a_map + 1], &full[slot], lk, tile.m0);
                    tma_load_2d(st + PAIR + A_BYTES, &maps[2 * sg.b_map + 1], &full[slot], lk,
                                tile.n0);
                }
                lk += BK;
            }
        }
        counts[0] = g;
    } else if (threadIdx.x == 32) {
        // MMA issuer: tile j of this CTA accumulates into TMEM columns (j & 1) * BNT
        int g = 0, j = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, ++j) {
            const tnk_gemm_task task = tasks[tiles[t].task];
            const int nk = ksteps(task);
            const int b = j & 1;
            if (j >= 2 && !mbar_wait_or_abort(&acc_empty[b], ((j >> 1) - 1) & 1, abort_flag)) {
                if (!*abort_flag) atomicExch(err, 13);
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + (uint32_t)(b * BNT);
            for (int i = 0; i < nk; ++i, ++g) {
                const int slot = g % STAGES;
                if (!mbar_wait_or_abort(&full[slot], (g / STAGES) & 1, abort_flag)) {
                    if (!*abort_flag) atomicExch(err, 11);
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                uint8_t* st = ring + slot * STAGE_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / 8; ++kk) {
                    const uint64_t ah = smem_desc(st + kk * 32);
                    const uint64_t bh = smem_desc(st + A_BYTES + kk * 32);
                    mma_tf32<BNT>(acc, ah, bh, (i > 0 || kk > 0) ? 1u : 0u);
                    if (PASSES == 3) {
                        const uint64_t al = smem_desc(st + PAIR + kk * 32);
                        const uint64_t bl = smem_desc(st + PAIR + A_BYTES + kk * 32);
                        mma_tf32<BNT>(acc, ah, bl, 1u);
                        mma_tf32<BNT>(acc, al, bh, 1u);
                    }
                }
                mma_commit(&empty[slot]);
            }
            if (ok) mma_commit(&acc_full[b]);      // arrives when this tile's MMAs are done
        }
        counts[1] = g;
        mma_commit(done);                          // arrives when every MMA issued is done
    } else if (warp >= 2) {
        // epilogue: TMEM lane quarter q = warp % 4 holds rows 32 q .. 32 q + 31 of the tile
        const int q = warp & 3;
        float* stg = stg_all + (warp - 2) * 32 * LDW;
        int j = 0;
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++j) {
            const tnk_gemm_tile tile = tiles[t];
            const tnk_gemm_task task = tasks[tile.task];
            const int nk = ksteps(task);
            const int b = j & 1;
            bool okw = true;
            if (lane == 0)
                okw = mbar_wait_or_abort(&acc_full[b], (j >> 1) & 1, abort_flag);
            okw = __shfl_sync(0xffffffffu, okw ? 1 : 0, 0) != 0;
            if (!okw) {
                if (lane == 0) {
                    if (!*abort_flag) atomicExch(err, 14);
                    *abort_flag = 1;
                }
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const bool f64 = (task.flags & 2) != 0;
            const int rows = min(32, task.m - (tile.m0 + q * 32));
            const int cols = min(BNT, task.n - tile.n0);
            for (int c0 = 0; c0 < BNT && c0 < cols; c0 += 32) {
                uint32_t v[32];
#pragma unroll
                for (int x = 0; x < 32; ++x) v[x] = 0u;
                if (nk > 0) {
                    const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) +
                                           (uint32_t)(b * BNT + c0);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
                          "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
                          "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                          "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
                          "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
                          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                          "=r"(v[30]), "=r"(v[31])
                        : "r"(taddr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                }
#pragma unroll
                for (int x = 0; x < 32; ++x) stg[lane * LDW + x] = __uint_as_float(v[x]);
                __syncwarp();
                const int64_t base =
                    task.c_off + (int64_t)(tile.m0 + q * 32) * task.ldc + tile.n0 + c0;
                if (f64)
                    store_rows<1>(reinterpret_cast<double*>(Cout), base, task.ldc, stg, LDW,
                                  rows, cols - c0, lane);
                else
                    store_rows<1>(reinterpret_cast<float*>(Cout), base, task.ldc, stg, LDW, rows,
                                  cols - c0, lane);
                __syncwarp();
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                 smem_u32(&acc_empty[b]))
                             : "memory");
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && *abort_flag) {
        for (int gg = counts[1]; gg < counts[0]; ++gg)
            mbar_wait(&full[gg % STAGES], (gg / STAGES) & 1);
    }
    if (threadIdx.x == 0 && !mbar_wait(done, 0)) atomicExch(err, 15);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(2 * BNT)
                     : "memory");
    }
}

constexpr size_t smem_bytes_p(int passes, int bn) {
    return 1024 + (size_t)stages_for(bn) * ((passes == 3) ? 2 : 1) * (TILE_BYTES + bn * BK * 4) +
           4 * 32 * 33 * 4 + 256;
}

constexpr size_t smem_bytes(int passes, int bn) {
    return 1024 + (size_t)stages_for(bn) * ((passes >= 3) ? 2 : 1) * (TILE_BYTES + bn * BK * 4) +
           256;
    // (1024: alignment slack of the ring; 256: barriers, TMEM slot, abort flag, counters)
}

template <int PASSES, int BNT>
int launch_tc_t(const tnk_gemm_task* tasks, const TcSeg* segs, const tnk_gemm_tile* tiles,
                int64_t n_tiles, const void* maps, void* C, int* err, cudaStream_t stream,
                bool pdl) {
    const size_t sm = smem_bytes(PASSES, BNT);
    cudaError_t e = cudaFuncSetAttribute(gemm_tc_kernel<PASSES, BNT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) {
        set_error("tc gemm: smem attribute: %s", cudaGetErrorString(e));
        return TNK_ERR_CUDA;
    }
    return launch_k("gemm_tc_kernel", gemm_tc_kernel<PASSES, BNT>, dim3((unsigned)n_tiles),
                    dim3(PASSES == 4 ? NT4 : NT), sm, stream, pdl, tasks, segs, tiles,
                    reinterpret_cast<const CUtensorMap*>(maps), C, err);
}

template <int PASSES, int BNT>
int launch_tc_persistent_t(const tnk_gemm_task* tasks, const TcSeg* segs,
                           const tnk_gemm_tile* tiles, int64_t n_tiles, int grid,
                           const void* maps, void* C, int* err, cudaStream_t stream, bool pdl) {
    const size_t sm = smem_bytes_p(PASSES, BNT);
    cudaError_t e = cudaFuncSetAttribute(gemm_tc_persistent_kernel<PASSES, BNT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) {
        set_error("tc gemm (persistent): smem attribute: %s", cudaGetErrorString(e));
        return TNK_ERR_CUDA;
    }
    return launch_k("gemm_tc_persistent_kernel", gemm_tc_persistent_kernel<PASSES, BNT>,
                    dim3((unsigned)grid), dim3(NT_P), sm, stream, pdl, tasks, segs, tiles,
                    (int)n_tiles, reinterpret_cast<const CUtensorMap*>(maps), C, err);
}

int g_tc_schedule = 0;       // 0: one tile per CTA; 1: persistent CTAs when tiles exceed SMs

int sm_count() {
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            n < 1)
            n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

}  // namespace

// bn: the tile width of this stage, 128 or 64; the B operand maps must have boxes of bn rows.
// pdl: launch as a programmatic dependent of the stream's previous kernel (launch_k).
int launch_gemm_tc(const tnk_gemm_task* tasks, const TcSeg* segs, const tnk_gemm_tile* tiles,
                   int64_t n_tiles, const void* maps, void* C, int* err, int passes, int bn,
                   cudaStream_t stream, bool pdl) {
    if (n_tiles < 0 || n_tiles > 0x7fffffff || (passes != 1 && passes != 3 && passes != 4) ||
        (bn != 128 && bn != 64)) {
        set_error("tc gemm: bad tile count %lld, passes %d or tile width %d", (long long)n_tiles,
                  passes, bn);
        return TNK_ERR_ARG;
    }
    if (n_tiles == 0) return TNK_OK;
    if (!tasks || !segs || !tiles || !maps || !C || !err) {
        set_error("tc gemm: null argument");
        return TNK_ERR_ARG;
    }
    if ((reinterpret_cast<uintptr_t>(maps) & 63) != 0) {
        set_error("tc gemm: tensor maps must be 64-byte aligned");
        return TNK_ERR_ARG;
    }
    const int nsm = sm_count();
    if (g_tc_schedule == 1 && n_tiles > nsm && passes != 4) {
        if (passes == 3)
            return bn == 128 ? launch_tc_persistent_t<3, 128>(tasks, segs, tiles, n_tiles, nsm,
                                                              maps, C, err, stream, pdl)
                             : launch_tc_persistent_t<3, 64>(tasks, segs, tiles, n_tiles, nsm,
                                                             maps, C, err, stream, pdl);
        return bn == 128 ? launch_tc_persistent_t<1, 128>(tasks, segs, tiles, n_tiles, nsm, maps,
                                                          C, err, stream, pdl)
                         : launch_tc_persistent_t<1, 64>(tasks, segs, tiles, n_tiles, nsm, maps,
                                                         C, err, stream, pdl);
    }
    if (passes == 4)
        return bn == 128
                   ? launch_tc_t<4, 128>(tasks, segs, tiles, n_tiles, maps, C, err, stream, pdl)
                   : launch_tc_t<4, 64>(tasks, segs, tiles, n_tiles, maps, C, err, stream, pdl);
    if (passes == 3)
        return bn == 128
                   ? launch_tc_t<3, 128>(tasks, segs, tiles, n_tiles, maps, C, err, stream, pdl)
                   : launch_tc_t<3, 64>(tasks, segs, tiles, n_tiles, maps, C, err, stream, pdl);
    return bn == 128 ? launch_tc_t<1, 128>(tasks, segs, tiles, n_tiles, maps, C, err, stream, pdl)
                     : launch_tc_t<1, 64>(tasks, segs, tiles, n_tiles, maps, C, err, stream, pdl);
}

// --------------------------------------------------------------------------------------------
// Tensor-map encoding (host): one 2-D map per staged operand block, FP32, box 32 x 128,
// SWIZZLE_128B, zero fill out of bounds. The driver entry point is looked up once.
// --------------------------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encoder() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

int encode_tmaps(const float* base, const int64_t* desc, int64_t n, void* out, int ncol) {
    EncodeTiledFn enc = get_encoder();
    if (!enc) {
        set_error("tensor maps: cuTensorMapEncodeTiled is unavailable");
        return TNK_ERR_DEVICE;
    }
    CUtensorMap* maps = reinterpret_cast<CUtensorMap*>(out);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t off = desc[ncol * i], rows = desc[ncol * i + 1],
                      cols = desc[ncol * i + 2], ld = desc[ncol * i + 3];
        const int64_t box_rows = ncol > 4 ? desc[ncol * i + 4] : BM;
        if (box_rows != 128 && box_rows != 64) {
            set_error("tensor map %lld: box rows %lld (128 or 64)", (long long)i,
                      (long long)box_rows);
            return TNK_ERR_ARG;
        }
        const float* p = base + off;
        if ((reinterpret_cast<uintptr_t>(p) & 15) != 0 || (ld * 4) % 16 != 0 || rows < 1 ||
            cols < 1 || ld < cols) {
            set_error("tensor map %lld: misaligned or bad extents (off %lld, ld %lld)",
                      (long long)i, (long long)off, (long long)ld);
            return TNK_ERR_ARG;
        }
        cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
        cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
        cuuint32_t box[2] = {BK, (cuuint32_t)box_rows};
        cuuint32_t estr[2] = {1, 1};
        CUresult r = enc(&maps[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)p, dims, strides,
                         box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            set_error("tensor map %lld: cuTensorMapEncodeTiled error %d", (long long)i, (int)r);
            return TNK_ERR_ARG;
        }
    }
    return TNK_OK;
}

}  // namespace tnk

// Selects how every later tensor-core GEMM stage is scheduled (process-wide): 0 = one CTA per
// tile, 1 = a persistent CTA per SM with two TMEM accumulators for stages with more tiles than
// SMs. Other values leave it unchanged. Returns the previous setting.
extern "C" int tnk_tc_schedule(int32_t mode) {
    const int prev = tnk::g_tc_schedule;
    if (mode == 0 || mode == 1) tnk::g_tc_schedule = mode;
    return prev;
}
