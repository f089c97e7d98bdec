/*
 * tnkit_gb300 -- C ABI of the GB300 (sm_103a) DMRG/TDVP inner-loop kernels.
 *
 * Every entry point takes raw device pointers, 64-bit sizes and a cudaStream_t (passed as
 * void*), launches asynchronously on that stream and returns an int status: TNK_OK (0) or a
 * positive TNK_ERR_* code; it never aborts. tnk_last_error() gives a message for the calling
 * thread's last failure. The library allocates no device memory on these paths: operands,
 * outputs, task tables and workspace are owned by the caller (torch in the Python host code).
 *
 * The H_eff matvec and the environment updates of the reference are each three stages over
 * charge blocks (dense tensors are the one-block case):
 *   stage 1  grouped GEMM   W1 = op(x_a) * op(x_b)         (one GEMM per output block)
 *   stage 2  combination    W2 = sum_t coef_t * W1[..]      (the MPO tensors, as scalars)
 *   stage 3  grouped GEMM   out = sum_seg W2 * op(x_c)      (segmented K over sectors)
 * The host builds the task tables of the three stages once per block layout from the
 * reference's block metadata (`Struct` offsets and shapes) and uploads them; the kernels then
 * read and write the reference's canonical flat block buffers in place.
 */
#ifndef TNKIT_GB300_H
#define TNKIT_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TNK_OK 0
#define TNK_ERR_ARG 1      /* a null pointer, a negative size, an unknown slot */
#define TNK_ERR_CUDA 2     /* a CUDA launch or runtime call failed */
#define TNK_ERR_SIZE 3     /* workspace or scratch too small for the plan */
#define TNK_ERR_DEVICE 4   /* set-up failed on the current device */

/* ----------------------------------------------------------------------------------------
 * Task tables (device arrays built by the host planner). Layouts are fixed by static
 * asserts in the .cu sources and by numpy dtypes in tnkit_gb300/plan.py.
 * ---------------------------------------------------------------------------------------- */

/* One output matrix of a grouped GEMM: C(i, j) at c_off + i*ldc + j, i < m, j < n.
 * C = sum over segments [seg_begin, seg_end) of coef * A_seg * B_seg; with no segment the
 * output is zero-filled. flags bit 0: accumulate into C instead of overwriting it; bit 1: FP64
 * output of a tensor-core stage; bit 2: output column stride 2 (one half of interleaved
 * complex128 data, C(i, j) at c_off + i*ldc + 2*j); bit 3: float-float output of a float-float
 * stage (a (hi, lo) float pair in each 8-byte element); bit 4: the task writes to the workspace
 * (operand slot 3) instead of C -- a split-K partial product summed by a plan's stage 4. */
typedef struct {
    int64_t c_off;
    int32_t ldc, m, n;
    int32_t seg_begin, seg_end;
    int32_t flags;
} tnk_gemm_task;                     /* 32 bytes */

/* One K segment: A(i, k) at buf[a_buf][a_off + i*a_rs + k*a_cs] (i < m, k < k_len),
 * B(k, j) at buf[b_buf][b_off + k*b_rs + j*b_cs]. Buffer slots are 0..3 (see below). */
typedef struct {
    int64_t a_off, b_off;
    int32_t a_rs, a_cs, b_rs, b_cs;
    int32_t k;
    int16_t a_buf, b_buf;
    int32_t conj;                    /* bit 0: conjugate A, bit 1: conjugate B (complex) */
    int32_t pad;
    double coef;
} tnk_gemm_seg;                      /* 56 bytes */

/* One output tile: task index and the tile's first row/column. The host lists the tiles of
 * every task, longest K first, so the block scheduler balances uneven sectors. */
typedef struct {
    int32_t task, m0, n0, pad;
} tnk_gemm_tile;                     /* 16 bytes */

/* Stage 2: dst(r, c) = sum over terms t of coef_t * src(r, c), r < rows, c < cols, with
 * dst(r, c) at dst_off + r*dst_ld + c*dst_cs and src(r, c) at src_off + r*src_ld + c*src_cs.
 * With no term the destination is zero-filled. */
typedef struct {
    int64_t dst_off;
    int32_t rows, cols, dst_ld, dst_cs;
    int32_t term_begin, term_end;
} tnk_comb_task;                     /* 32 bytes */

typedef struct {
    int64_t src_off;
    int32_t src_ld, src_cs;
    double coef;
} tnk_comb_term;                     /* 24 bytes */

/* A chunk of rows [row0, row1) of one combination task: the launch grid. */
typedef struct {
    int32_t task, row0, row1, pad;
} tnk_comb_item;                     /* 16 bytes */

/* A three-stage contraction plan: device pointers to the tables above and their counts, plus
 * the workspace it needs (elements of the stage-1 and stage-2 intermediates). Plain data,
 * filled by the host; the library keeps no reference to it after a call returns. */
typedef struct {
    const tnk_gemm_task* t1; const tnk_gemm_seg* s1; const tnk_gemm_tile* tiles1; int64_t n_tiles1;
    const tnk_comb_task* t2; const tnk_comb_term* c2; const tnk_comb_item* items2; int64_t n_items2;
    const tnk_gemm_task* t3; const tnk_gemm_seg* s3; const tnk_gemm_tile* tiles3; int64_t n_tiles3;
    int64_t ws1_elems;               /* stage-1 output: workspace elements [0, ws1_elems) */
    int64_t ws2_elems;               /* stage-2 output and split-K partials:
                                        [ws1_elems, ws1_elems + ws2_elems) */
    int64_t out_elems;               /* elements of the output buffer */
    /* optional stage 4: the stage-3 tasks split along K (flags bit 4) write partial products to
     * the workspace; this combination sums them, in a fixed order, into the output */
    const tnk_comb_task* t4; const tnk_comb_term* c4; const tnk_comb_item* items4; int64_t n_items4;
} tnk_plan3;

/* ----------------------------------------------------------------------------------------
 * Library information
 * ---------------------------------------------------------------------------------------- */
const char* tnk_version(void);
const char* tnk_last_error(void);
/* Sizes of the table structs above, so a binding can check its own layout. */
int tnk_struct_sizes(int64_t* out6);

/* ----------------------------------------------------------------------------------------
 * The hot path: H_eff matvecs and environment updates (FP64)
 *
 * Operand slots of a plan3: slot 0 = x0, slot 1 = x1, slot 2 = x2, slot 3 = the workspace.
 * `ws` holds ws1_elems + ws2_elems doubles. All buffers are the reference's canonical flat
 * block buffers (tnkit/blocks.py:243-252) or, for dense tensors, C-contiguous arrays.
 * ---------------------------------------------------------------------------------------- */

/* Generic three-stage contraction. */
int tnk_contract3_f64(const tnk_plan3* plan, const double* x0, const double* x1,
                      const double* x2, double* out, double* ws, int64_t ws_elems,
                      void* stream);

/* (H_eff theta) for two sites: out[p,s,t,d] = sum L[p,w,q] th[q,i,j,b] W1[w,m,s,i]
 * W2[m,r,t,j] R[d,r,b]. Replaces tnkit/_dmrg.py:162-169 (apply_two_site) and, for dense
 * tensors, :172-189 (fused_two_site + apply_two_site_fused). W1, W2 are folded into the plan.
 * x0 = L, x1 = theta, x2 = R. */
int tnk_apply_two_site_f64(const tnk_plan3* plan, const double* L, const double* theta,
                           const double* R, double* out, double* ws, int64_t ws_elems,
                           void* stream);

/* (H_eff M) for one site. Replaces tnkit/_dmrg.py:192-199 (apply_one_site). */
int tnk_apply_one_site_f64(const tnk_plan3* plan, const double* L, const double* M,
                           const double* R, double* out, double* ws, int64_t ws_elems,
                           void* stream);

/* L'[d,r,e] = sum L[p,w,q] conj(A[p,s,d]) W[w,r,s,y] A[q,y,e].
 * Replaces tnkit/_dmrg.py:216-222 (update_left_env). x0 = A (read twice), x1 = L. */
int tnk_update_left_env_f64(const tnk_plan3* plan, const double* L, const double* A,
                            double* out, double* ws, int64_t ws_elems, void* stream);

/* R'[u,w,v] = sum R[x,r,y] conj(B[u,s,x]) W[w,r,s,p] B[v,p,y].
 * Replaces tnkit/_dmrg.py:225-231 (update_right_env). x0 = B (read twice), x1 = R. */
int tnk_update_right_env_f64(const tnk_plan3* plan, const double* R, const double* B,
                             double* out, double* ws, int64_t ws_elems, void* stream);

/* The two-site matvec above for callers that cannot allocate device memory (code in a host
 * callback or signal-safe section, a fixed pre-sized memory pool, an embedding or binding with
 * no device allocator): no counterpart in the reference. Instead of a caller workspace it uses
 * one fixed scratch array in the library's device memory, TNK_NOALLOC_SCRATCH_ELEMS doubles
 * (64 MiB, enough for the chi=1024 U(1) XXZ mid bond, which needs 7.9 M), held on every GPU that
 * loads the library until the process exits. Plans needing more scratch get TNK_ERR_SIZE. The
 * first call on each device looks up the array's device address (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture. The address is cached for the
 * process: after a cudaDeviceReset of that device it is stale, so do not call this entry point on
 * a device that was reset. All calls share the array, so calls that overlap on the GPU race;
 * order them on one stream. Allocates nothing. */
#define TNK_NOALLOC_SCRATCH_ELEMS 8388608
int tnk_apply_two_site_f64_noalloc(const tnk_plan3* plan, const double* L, const double* theta,
                                   const double* R, double* out, void* stream);
/* out[0] = TNK_NOALLOC_SCRATCH_ELEMS, as compiled into the library. */
int tnk_noalloc_scratch_elems(int64_t* out);

/* The same plans in float-float ("double-FP32") arithmetic on the FP32 CUDA cores: operands
 * are (hi, lo) float pairs (48 significant bits) stored in buffers with the FP64 layout, products
 * by error-free transformations; ~1e-13 relative on the H_eff contractions at several times the
 * FP64 rate of GB300. Stage-1 tasks carry flags bit 3 (float-float intermediates), GEMM segment
 * coefficients must be +1 or -1. Replaces the same reference functions as the FP64 entry points.
 * tnk_ff_split: y[i] = (fl(x[i]), fl(x[i] - fl(x[i]))) for n doubles (y may not alias x). */
int tnk_ff_split(const double* x, double* y, int64_t n, void* stream);
/* x0..x2 already split (float-float buffers); out is float-float where a task says so. */
int tnk_contract3_ff(const tnk_plan3* plan, const double* x0, const double* x1,
                     const double* x2, double* out, double* ws, int64_t ws_elems, void* stream);
/* L2, R2: float-float copies (tnk_ff_split) of L and R; theta, out: FP64. `ws` holds
 * ws1_elems + ws2_elems + out_elems doubles (the split theta goes after the intermediates). */
int tnk_apply_two_site_ff(const tnk_plan3* plan, const double* L2, const double* theta,
                          const double* R2, double* out, double* ws, int64_t ws_elems,
                          void* stream);
int tnk_grouped_gemm_ff(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                        const tnk_gemm_tile* tiles, int64_t n_tiles, const double* b0,
                        const double* b1, const double* b2, const double* b3, double* C,
                        void* stream);

/* The inner product of the FP64 grouped GEMM kernel behind every FP64 entry point, process-wide:
 * 0 = per-thread FP64 FMAs (4 x 4 register tile), 1 = FP64 tensor MMAs (mma.sync m8n8k4,
 * 8 x 8 tiles per warp instruction). Same tables, loaders and results (to rounding). Any other
 * value leaves the setting unchanged. Returns the previous setting. No counterpart in the
 * reference (it calls cuBLAS through torch). */
int tnk_gemm_f64_variant(int32_t variant);

/* One grouped GEMM stage on its own (a two-operand block contraction, e.g. theta = M_i M_i+1,
 * tnkit/blocks.py:1156-1192 tensordot). Slots 0..3 = b0..b3; C is the output base. */
int tnk_grouped_gemm_f64(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                         const tnk_gemm_tile* tiles, int64_t n_tiles, const double* b0,
                         const double* b1, const double* b2, const double* b3, double* C,
                         void* stream);

/* One combination stage on its own: block gathers, fuse and split of legs
 * (tnkit/blocks.py:755-760, :822-838) are combinations with one unit term per piece. */
int tnk_combine_f64(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                    const tnk_comb_item* items, int64_t n_items, const double* src,
                    double* dst, void* stream);

/* ----------------------------------------------------------------------------------------
 * Mixed precision: the two-site matvec on the tcgen05 tensor cores (TF32 inputs, FP32
 * accumulation in TMEM), FP64 in and out. Replaces, for the bulk Lanczos iterations, the
 * low-precision matvec of tnkit/_dmrg.py:691-695 (eig='lanczos-mixed', there complex64 einsums).
 * passes = 3 splits every operand into TF32 hi/lo parts (~1e-6 relative error); passes = 1 is
 * plain TF32 (~1e-3); passes = 4 is passes 3 with the operands staged once as FP32 and the hi/lo
 * parts formed in shared memory inside the GEMM (half the operand traffic, the same accuracy).
 * ---------------------------------------------------------------------------------------- */

/* A tensor-core GEMM segment: operand tensor maps (hi parts at index 2*map, lo at 2*map+1). */
typedef struct {
    int32_t a_map, b_map, k, pad;
} tnk_tc_seg;                        /* 16 bytes */

/* Staging of one FP64 block into the FP32 operand layout: source rows x cols (row stride
 * src_ld) -> destination (transposed when `transpose`: cols x rows) with row stride dst_ld. */
typedef struct {
    int64_t src_off, dst_off;
    int32_t rows, cols, src_ld, dst_ld;
    int32_t transpose, pad;
} tnk_cvt_task;                      /* 40 bytes */

typedef struct {
    int32_t task, r0, c0, pad;       /* one 32 x 32 source tile */
} tnk_cvt_item;                      /* 16 bytes */

/* The tensor-core two-site plan. `stage` is one FP32 buffer holding every staged operand (L, R,
 * theta^T, Z) at the tables' offsets, hi parts first and lo parts at +lo_off; `y32` holds the
 * stage-1 output. `maps` are the CUtensorMaps (128 bytes each, 64-byte aligned) of the staged
 * blocks; `err` is a device word that a kernel sets (nonzero) if a bounded wait timed out.
 * bn3: the tile width of stage 3 (128 x bn3 tiles; 0 means 128, or 64, in which case the maps
 * of stage 3's B operands must have boxes of 64 rows, tnk_tc_encode_tmaps_box). */
typedef struct {
    const tnk_cvt_task* cvt; const tnk_cvt_item* cvt_items; int64_t n_cvt_items;
    const tnk_gemm_task* t1; const tnk_tc_seg* s1; const tnk_gemm_tile* tiles1; int64_t n_tiles1;
    const tnk_comb_task* t2; const tnk_comb_term* c2; const tnk_comb_item* items2; int64_t n_items2;
    const tnk_gemm_task* t3; const tnk_tc_seg* s3; const tnk_gemm_tile* tiles3; int64_t n_tiles3;
    const void* maps;
    float* stage; int64_t lo_off;
    float* y32;
    int* err;
    int32_t passes, bn3;
} tnk_tc_plan;

/* out = H_eff theta (FP64 canonical buffers) through the tensor cores: stage theta, two tcgen05
 * grouped GEMMs around the FP32 MPO combination. L and R must have been staged into the plan's
 * buffer with tnk_stage_f32 (once per local problem). */
int tnk_apply_two_site_tc(const tnk_tc_plan* plan, const double* theta, double* out,
                          void* stream);
/* Stage FP64 blocks into FP32 (split into hi/lo parts when `split`). */
int tnk_stage_f32(const tnk_cvt_task* tasks, const tnk_cvt_item* items, int64_t n_items,
                  const double* src, float* dst, int64_t lo_off, int32_t split, void* stream);
/* Encode n 2-D FP32 tensor maps (host side; needs the CUDA driver): desc4 holds (element offset
 * from `base`, rows, cols, row stride) per map; out receives n * 128 bytes. */
int tnk_tc_encode_tmaps(const float* base, const int64_t* desc4, int64_t n, void* out);
/* The same with a fifth column per map: the box rows (128, or 64 for the B operands of a stage
 * run with 128 x 64 tiles). */
int tnk_tc_encode_tmaps_box(const float* base, const int64_t* desc5, int64_t n, void* out);
/* One tensor-core grouped GEMM stage (flags bit 1 of a task: FP64 output, else FP32). */
int tnk_grouped_gemm_tc(const tnk_gemm_task* tasks, const tnk_tc_seg* segs,
                        const tnk_gemm_tile* tiles, int64_t n_tiles, const void* maps, void* C,
                        int* err, int32_t passes, void* stream);
/* How tensor-core GEMM stages are scheduled from now on, process-wide: 0 = one CTA per output
 * tile; 1 = stages with more tiles than SMs run one persistent CTA per SM with two TMEM
 * accumulators (the epilogue of one tile under the MMAs of the next). Other values leave the
 * setting unchanged; returns the previous one. No counterpart in the reference. */
int tnk_tc_schedule(int32_t mode);
/* The same with 128 x bn tiles (bn = 128 or 64; B maps with boxes of bn rows). */
int tnk_grouped_gemm_tc_bn(const tnk_gemm_task* tasks, const tnk_tc_seg* segs,
                           const tnk_gemm_tile* tiles, int64_t n_tiles, const void* maps,
                           void* C, int* err, int32_t passes, int32_t bn, void* stream);
/* Stage 2 on FP32 data (hi/lo split of the result when `split`). */
int tnk_combine_f32(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                    const tnk_comb_item* items, int64_t n_items, const float* src, float* dst,
                    int64_t lo_off, int32_t split, void* stream);

/* ----------------------------------------------------------------------------------------
 * Lanczos vector kernels (FP64). Replace the reductions and CGS2 reorthogonalisation of
 * tnkit/eigensolver.py:560-604 (vdot, norm, two classical Gram-Schmidt passes).
 * `red` is a caller workspace of at least TNK_RED_ELEMS doubles (16-byte aligned) for the
 * reductions;
 * results are written to device memory, so no call synchronises.
 * ---------------------------------------------------------------------------------------- */
#define TNK_RED_ELEMS 65536

/* out[0] = sum_k x[k] y[k] (deterministic order). */
int tnk_dot_f64(const double* x, const double* y, int64_t n, double* out, double* red,
                void* stream);
/* out[0] = ||x||_2. */
int tnk_nrm2_f64(const double* x, int64_t n, double* out, double* red, void* stream);
/* c[i] = sum_k V[i*ldv + k] w[k], i < nv (nv <= 64). */
int tnk_multidot_f64(const double* V, int64_t ldv, int32_t nv, const double* w, int64_t n,
                     double* c, double* red, void* stream);
/* w[k] = w[k] - sum_i c[i] V[i*ldv + k], with c on the device (nv <= 64). */
int tnk_gemv_sub_f64(const double* V, int64_t ldv, int32_t nv, const double* c, double* w,
                     int64_t n, void* stream);
/* One fused pass of classical Gram-Schmidt against the rows V[0..nv) (nv <= 64), over a single
 * read of the basis; `mode` is a sum of
 *   TNK_CGS_SUB  w[k] -= sum_i cin[i] V[i*ldv + k]      (cin on the device; i ascending)
 *   TNK_CGS_DOT  out[i] = sum_k V[i*ldv + k] w[k], i < nv (w after the subtraction)
 *   TNK_CGS_NRM  out[0] = ||w||_2                        (w after the subtraction)
 * (DOT and NRM exclude each other). Two passes, SUB|DOT then SUB|NRM after a DOT, are CGS2 with
 * the Lanczos coefficients alpha = c1[j] + c2[j] and beta = ||w|| (the reference computes the
 * same numbers with a three-term step, tnkit/eigensolver.py:567-599). The reduction finishes
 * inside the launch: `counter` is a zero-initialised uint32 in device memory, used by one
 * stream at a time, and left zero on return; `red` holds TNK_RED_ELEMS doubles, 16-byte
 * aligned. */
#define TNK_CGS_SUB 1
#define TNK_CGS_DOT 2
#define TNK_CGS_NRM 4
int tnk_cgs_pass_f64(const double* V, int64_t ldv, int32_t nv, const double* cin, double* w,
                     int64_t n, double* out, int32_t mode, double* red, uint32_t* counter,
                     void* stream);
/* The same pass over many independent vectors concatenated in one batch vector (the chains of
 * a batched Lanczos): chain c occupies [off[c], off[c+1]) of w and of every basis row (ldv = the
 * batch length); the chains ids[0..nseg) are processed in one launch, each with its own
 * coefficients cin + c*rec_stride, output out + c*rec_stride and completion counter counter[y]
 * (y = its position in ids; zero before the call, left zero). max_len >= the longest listed
 * segment; nseg * 66 <= TNK_RED_ELEMS (66 partial doubles per CTA). off and ids are device arrays. No
 * reduction mixes chains: each chain's results equal tnk_cgs_pass_f64 on its segment up to the
 * order of its partial sums. Replaces the per-chain passes of a batched solve (the reference
 * runs one chain per call, its CGS2 at tnkit/eigensolver.py:567-599). */
int tnk_cgs_pass_seg_f64(const double* V, int64_t ldv, int32_t nv, const double* cin, double* w,
                         const int64_t* off, const int32_t* ids, int32_t nseg, int64_t max_len,
                         int64_t rec_stride, double* out, int32_t mode, double* red,
                         uint32_t* counter, void* stream);
/* y_c = x_c * (f / s[c * s_stride]) on the segments [off[c], off[c+1]) of the chains
 * ids[0..nseg) (device arrays), max_len >= the longest: the per-chain normalisation of a
 * batched Lanczos step in one launch (the reference: one chain's `w / beta`,
 * tnkit/eigensolver.py:600-604). */
int tnk_scale_div_seg_f64(const double* x, double* y, const int64_t* off, const int32_t* ids,
                          int32_t nseg, int64_t max_len, const double* s, int64_t s_stride,
                          double f, void* stream);
/* The same pass on FP32 vectors (FP32 arithmetic; coefficients and results in double): the
 * Krylov basis of the tensor-core stage of the mixed-precision solve, whose operator is only
 * ~1e-6 accurate, is kept in FP32. */
int tnk_cgs_pass_f32(const float* V, int64_t ldv, int32_t nv, const double* cin, float* w,
                     int64_t n, double* out, int32_t mode, double* red, uint32_t* counter,
                     void* stream);
/* y = x * (f / s[0]) on FP32 vectors, s on the device (double). */
int tnk_scale_div_f32(const float* x, float* y, int64_t n, const double* s, double f,
                      void* stream);
/* Thick-restart rotation of an FP32 basis: out[q*ldo + k] = sum_r Y[r*kk + q] V[r*ldv + k] for
 * q < kk, r < nv (nv, kk <= 64; Y row-major nv x kk doubles on the device, used in FP32; out must
 * not overlap V). Replaces the (kk x cur)(cur x n) product U = Yk^T Vb[:cur] of the reference's
 * restart, tnkit/eigensolver.py:626-636. */
int tnk_rotate_f32(const float* V, int64_t ldv, int32_t nv, const double* Y, int32_t kk,
                   float* out, int64_t ldo, int64_t n, void* stream);
/* y = a*x + b*y with the scalars a = sa[0]*fa, b = sb[0]*fb read from device memory when
 * sa/sb are non-null (else 1): lets Lanczos use alpha/beta without a host round trip. */
int tnk_axpby_f64(const double* x, double* y, int64_t n, const double* sa, double fa,
                  const double* sb, double fb, void* stream);
/* y = x * (f / s[0]) (normalisation by a device scalar). */
int tnk_scale_div_f64(const double* x, double* y, int64_t n, const double* s, double f,
                      void* stream);

/* ----------------------------------------------------------------------------------------
 * Complex128 Lanczos kernels (interleaved re/im doubles; n counts complex entries). They serve
 * the Krylov exponential of two-site TDVP (tnkit/eigensolver.py:282-349, block twin
 * tnkit/block_lanczos.py:76-121): vdot conjugates its first argument, as the reference's does.
 * Complex matvecs and environment updates use the FP64 entry points above on plans whose
 * segments and outputs address the real and imaginary halves separately (flags bit 2).
 * ---------------------------------------------------------------------------------------- */
/* out[0] + i out[1] = sum_k conj(x[k]) y[k]. */
int tnk_zdot_f64(const double* x, const double* y, int64_t n, double* out, double* red,
                 void* stream);
/* c[i] = sum_k conj(V[i*ldv + k]) w[k], i < nv <= 64 (c: 2*nv doubles). */
int tnk_zmultidot_f64(const double* V, int64_t ldv, int32_t nv, const double* w, int64_t n,
                      double* c, double* red, void* stream);
/* w[k] -= sum_i c[i] V[i*ldv + k], complex c on the device. */
int tnk_zgemv_sub_f64(const double* V, int64_t ldv, int32_t nv, const double* c, double* w,
                      int64_t n, void* stream);
/* y = a x + b y, a = sa[0]*fa, b = sb[0]*fb with complex sa, sb on the device (1 when null). */
int tnk_zaxpby_f64(const double* x, double* y, int64_t n, const double* sa, double fa,
                   const double* sb, double fb, void* stream);

/* Eigenvalues (ascending) and eigenvectors of `batch` real symmetric tridiagonal matrices of
 * order n <= TNK_TRIDIAG_MAX_N, on the device: matrix b has diagonal d[b*ld_d + i] and
 * off-diagonal e[b*ld_e + i] (i < n - 1); lam[b*n + j] and column j of the row-major n x n
 * V[b*n*n ...] are its j-th eigenpair. Implicit QL with Wilkinson-type shifts, one thread block
 * per matrix; info[b] = 0, or the index + 1 of an eigenvalue that did not converge. Replaces the
 * tridiagonal eigensolve of the reference's Krylov exponential, expm_sym_tridiag_eigh(_batched)
 * (tnkit/backend.py:643-661, :729-751), whose torch.linalg.eigh it computes. */
#define TNK_TRIDIAG_MAX_N 128
int tnk_tridiag_eig_f64(const double* d, const double* e, int64_t n, int64_t batch,
                        int64_t ld_d, int64_t ld_e, double* lam, double* V, int32_t* info,
                        void* stream);

/* ----------------------------------------------------------------------------------------
 * Truncation: the per-sector factorisation of tnkit/blocks.py:1380-1462 with method='gram'
 * (the block SVD through the smaller Gram matrix, tnkit/blocks.py:1345-1377) on cuSOLVER and
 * cuBLAS. M is a row-major R x C block; U (R x k) and Vh (k x C) are written row-major, S (k)
 * descending (stable order), k = min(R, C). The call synchronises its stream and returns when
 * the outputs are written; S_host (optional, k doubles) receives a host copy of S. It allocates
 * nothing: `ws` (256-byte aligned) holds at least tnk_svd_gram_ws_f64(R, C) bytes. Calls on
 * different streams from different host threads run concurrently (handles are per thread).
 * ---------------------------------------------------------------------------------------- */
int tnk_svd_gram_ws_f64(int64_t R, int64_t C, int64_t* bytes);
int tnk_svd_gram_f64(const double* M, int64_t R, int64_t C, double* U, double* S, double* Vh,
                     void* ws, int64_t ws_bytes, double* S_host, void* stream);
/* The same with the side the sweep keeps canonical taken straight from its own Gram matrix
 * (no QR): orth = 1 gives U orthonormal (eigenvectors of M M^T) and Vh = diag(1/S) U^T M,
 * orth = 2 gives Vh orthonormal (eigenvectors of M^T M) and U = M V diag(1/S), with
 * S = sqrt(max(lambda, 0)) descending; orth = 0 is tnk_svd_gram_f64. */
int tnk_svd_gram_ws2_f64(int64_t R, int64_t C, int32_t orth, int64_t* bytes);
int tnk_svd_gram2_f64(const double* M, int64_t R, int64_t C, int32_t orth, double* U,
                      double* S, double* Vh, void* ws, int64_t ws_bytes, double* S_host,
                      void* stream);
/* The same in FP32 (S_host still double): the truncations of the opening sweeps of the mixed
 * schedule, whose local solves are only tensor-core accurate. */
int tnk_svd_gram_ws_f32(int64_t R, int64_t C, int64_t* bytes);
int tnk_svd_gram_f32(const float* M, int64_t R, int64_t C, float* U, float* S, float* Vh,
                     void* ws, int64_t ws_bytes, double* S_host, void* stream);

/* The O(n^3) steps of the same Gram eigh for all sectors of a bond at once (the per-sector eigh
 * of tnkit/blocks.py:1345-1377 inside the truncation of tnkit/blocks.py:1380-1462), hand-written
 * for the device: the Householder reduction of every sector's Gram matrix to tridiagonal form in
 * one launch (one thread-block cluster of `cluster` CTAs per sector, the matrix resident in the
 * cluster's distributed shared memory), and the back-transformation U = Q Z of the tridiagonal
 * eigenvectors Z that the cut keeps, in one launch. Between them, the caller solves the
 * tridiagonal eigenproblems (d, e). Sector s: order n, its Gram matrix at G + g_off (n x n,
 * column-major; the lower triangle is read), its d, e, tau at + v_off (n entries each; e and tau
 * use n - 1), its Z at Z + z_off (column-major n x k, ld n). On return from the reduction,
 * column k of G holds reflector k's v in rows k+1 .. n-1 (v[k+1] = 1). The table arrays are
 * device memory; the calls only enqueue work on `stream`. */
typedef struct {
    int64_t n, g_off, v_off, z_off;
} tnk_sytrd_sector;
typedef struct {
    int32_t sector, col0, ncols, pad;    /* ncols <= 8 columns of one sector's Z */
} tnk_ormtr_item;
/* The largest order the reduction takes with clusters of `cluster` (1, 2, 4, 8, 16) CTAs on
 * the current device; 0 when such clusters cannot be launched there. */
int tnk_sytrd_limits(int32_t cluster, int32_t* n_max);
/* n_max: the largest n of the batch (at most tnk_sytrd_limits(cluster)). */
int tnk_sytrd_batched_f64(const tnk_sytrd_sector* sectors, int32_t n_sectors, int32_t n_max,
                          int32_t cluster, double* G, double* d, double* e, double* tau,
                          void* stream);
int tnk_ormtr_batched_f64(const tnk_sytrd_sector* sectors, const tnk_ormtr_item* items,
                          int32_t n_items, int32_t n_max, const double* G, const double* tau,
                          double* Z, void* stream);

/* The O(n^3) steps of the exact per-sector SVD of the truncation (method='svd', the reference's
 * default, tnkit/blocks.py:1310-1344 inside :1380-1462) for all sectors of a bond at once: the
 * Householder bidiagonalisation A = Q_L B Q_R^T of every sector's m x n working matrix (m >= n:
 * the block, or its transpose) in one launch (one thread-block cluster per sector, the matrix
 * resident in the cluster's distributed shared memory), and the back-transformations of the
 * singular vectors the cut keeps (tnk_ormqr_batched_f64). Between them, the caller solves the
 * bidiagonal SVDs (d, e). Sector s: A(i, j) = M[a_off + i a_rs + j a_cs]; its left reflectors
 * (column k: u_k in rows k .. m-1, u_k[k] = 1) into the m x n column-major matrix at
 * UL + ul_off, its right reflectors (column k: v_k in rows k+1 .. n-1, v_k[k+1] = 1) into the
 * n x n column-major matrix at VR + vr_off, and d (n), e (n - 1), tau_u (n), tau_v (n - 2) at
 * vec + v_off + {0, n, 2n, 3n}. Tables are device memory; the calls only enqueue work. */
typedef struct {
    int64_t m, n, a_off, ul_off, vr_off, v_off, spare;
    int32_t a_rs, a_cs;
} tnk_gebrd_sector;                  /* 64 bytes */
/* Z <- H_0 H_1 ... H_{nrefl-1} Z: reflector k in column k of the rows x nrefl column-major
 * matrix at R + r_off, from row k + shift (that entry 1) to rows - 1, its tau at
 * tau + tau_off + k; Z column-major rows x (columns named by the items), at Z + z_off. */
typedef struct {
    int64_t rows, nrefl, r_off, tau_off, z_off;
    int32_t shift, pad;
} tnk_refl_set;                      /* 48 bytes */
/* The largest m (with n <= m) the bidiagonalisation takes with clusters of `cluster` CTAs on
 * the current device; 0 when such clusters cannot be launched there. */
int tnk_gebrd_limits(int32_t cluster, int32_t* m_max);
int tnk_gebrd_batched_f64(const tnk_gebrd_sector* sectors, int32_t n_sectors, int32_t m_max,
                          int32_t n_max, int32_t cluster, const double* M, double* UL,
                          double* VR, double* vec, void* stream);
int tnk_ormqr_batched_f64(const tnk_refl_set* sets, const tnk_ormtr_item* items,
                          int32_t n_items, int32_t rows_max, const double* R, const double* tau,
                          double* Z, void* stream);

/* ----------------------------------------------------------------------------------------
 * Host planner: the block tables of the one- and two-site H_eff contraction (the stage-1 /
 * stage-2 / stage-3 tables above) built natively from the layouts' sector keys, and their
 * re-layout for the tensor-core path. It replaces the block pairing that the reference does in
 * Python at every tensordot (tnkit/blocks.py:1089-1090, per pair of matching blocks) with one
 * pass over the keys per local problem. Host memory only; no CUDA call.
 * ---------------------------------------------------------------------------------------- */
typedef struct {
    int32_t nlegs, nblocks;
    const int64_t* keys;             /* nblocks x nlegs sector indices (canonical order) */
    const int64_t* shapes;           /* nblocks x nlegs block extents */
    const int64_t* offsets;          /* nblocks element offsets */
} tnk_layout_desc;

typedef struct {
    int32_t n_sites, pad;            /* 1 or 2 */
    tnk_layout_desc theta;           /* (a, s_1 .. s_n, b) */
    tnk_layout_desc L;               /* (a', w, a) */
    tnk_layout_desc R;               /* (b', r, b) */
    tnk_layout_desc out;             /* (a', s'_1 .. s'_n, b') */
    const double* S;                 /* combined MPO, dense C order over the axes
                                        (w, in_1 .. in_n, out_1 .. out_n, r) */
    int64_t s_dims[6];               /* its extents (2 n + 2 used) */
    const int64_t* sec_start;        /* sector starts along the axes of S, axis by axis */
    const int64_t* sec_dim;          /* and their extents */
    int64_t sec_begin[7];            /* axis a's sectors at [sec_begin[a], sec_begin[a + 1]) */
} tnk_apply_plan_in;

/* Environment-update plan: side 0 builds L'[d,r,e] = sum L[p,w,q] conj(A[p,s,d]) W[w,r,s,y]
 * A[q,y,e] (env = L, site = A), side 1 builds R'[u,w,v] = sum R[x,r,y] conj(B[u,s,x])
 * W[w,r,s,p] B[v,p,y] (env = R, site = B); W is the dense MPO tensor over its sector-ordered
 * indices with the sector starts / extents of its four legs. Tables 0 .. 5 as for the H_eff
 * plan (stage-1 GEMMs: conj(site) x env; stage 2: MPO coefficients; stage 3: x site). */
typedef struct {
    int32_t side, pad;
    tnk_layout_desc env;
    tnk_layout_desc site;
    tnk_layout_desc out;
    const double* W;
    int64_t w_dims[4];
    const int64_t* sec_start;
    const int64_t* sec_dim;
    int64_t sec_begin[5];
} tnk_env_plan_in;

int tnk_env_plan_build(const tnk_env_plan_in* in, void** handle);
/* Block tensordot plan: out = a . b contracting the last nc legs of a with the first nc legs
 * of b (out's layout given: the free legs of a, then those of b); tables 0 / 1 hold one GEMM task
 * per output block and one K segment per matching block pair (slots x0 = a, x1 = b). */
int tnk_tensordot_plan_build(const tnk_layout_desc* a, const tnk_layout_desc* b,
                             const tnk_layout_desc* out, int32_t nc, void** handle);

/* Tables of a built plan, read back with tnk_planb_table(handle, id, &data, &count):
 * 0 stage-1 tasks, 1 stage-1 segments, 2 stage-2 tasks, 3 stage-2 terms, 4 stage-3 tasks,
 * 5 stage-3 segments (tnk_apply_plan_build); 10 stage-1 tasks, 11 stage-1 tensor-core segments,
 * 12 stage-2 tasks, 13 stage-3 tasks, 14 stage-3 tensor-core segments, 15 tensor maps
 * (int64 offset, rows, cols, ld each), 16 / 17 / 18 the staging tasks of L / R / theta
 * (tnk_plan_tc_build). tnk_planb_scalars: ws1, ws2, stage-1 MACs, stage-3 MACs, staging
 * elements. */
int tnk_apply_plan_build(const tnk_apply_plan_in* in, void** handle);
int tnk_plan_tc_build(const tnk_gemm_task* t1, int64_t nt1, const tnk_gemm_seg* s1,
                      const tnk_comb_task* t2, int64_t nt2, const tnk_gemm_task* t3,
                      int64_t nt3, const tnk_gemm_seg* s3, void** handle);
/* Stage 3's long tasks cut along K so that one wave of tiles finishes together: a task whose
 * tile work (K x min(tile_m, m) x min(tile_n, n)) exceeds the average work per resident CTA
 * (slots) is split into at most max_chunks chunks writing compact partials at ws_base + ...
 * (flags bit 4); tables 4 / 5 hold the new stage-3 tasks and segments, 2 / 3 the stage-4
 * combination summing the partials in chunk order; scalars: 1 when anything was split (else
 * the tables are empty and the input stands), then the workspace elements added. */
int tnk_plan_split_k(const tnk_gemm_task* t, int64_t nt, const tnk_gemm_seg* s, int64_t ws_base,
                     int32_t slots, int32_t max_chunks, int32_t tile_m, int32_t tile_n,
                     void** handle);
int tnk_planb_table(const void* handle, int32_t id, const void** data, int64_t* count);
int tnk_planb_scalars(const void* handle, int64_t* out5);
void tnk_planb_free(void* handle);

#ifdef __cplusplus
}
#endif
#endif /* TNKIT_GB300_H */
