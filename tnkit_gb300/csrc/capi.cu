// extern "C" entry points of libtnkit_gb300 (declared in include/tnkit_gb300.h).
#include <stdarg.h>
#include <string.h>

#include "tnk_internal.cuh"

namespace tnk {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int vec_dot(const double*, const double*, int64_t, double*, double*, int, cudaStream_t);
int vec_multidot(const double*, int64_t, int, const double*, int64_t, double*, double*,
                 cudaStream_t);
int vec_gemv_sub(const double*, int64_t, int, const double*, double*, int64_t, cudaStream_t);
int vec_axpby(const double*, double*, int64_t, const double*, double, const double*, double,
              cudaStream_t);
int vec_scale_div(const double*, double*, int64_t, const double*, double, cudaStream_t);
int vec_cgs_pass(const double*, int64_t, int, const double*, double*, int64_t, double*, int,
                 double*, unsigned*, cudaStream_t);
int vec_scale_div_seg(const double*, double*, const int64_t*, const int32_t*, int, int64_t,
                      const double*, int64_t, double, cudaStream_t);
int vec_cgs_pass_seg(const double*, int64_t, int, const double*, double*, const int64_t*,
                     const int32_t*, int, int64_t, int64_t, double*, int, double*, unsigned*,
                     cudaStream_t);
int vec_cgs_pass_f32(const float*, int64_t, int, const double*, float*, int64_t, double*, int,
                     double*, unsigned*, cudaStream_t);
int vec_scale_div_f32(const float*, float*, int64_t, const double*, double, cudaStream_t);
int vec_rotate_f32(const float*, int64_t, int, const double*, int, float*, int64_t, int64_t,
                   cudaStream_t);

// The three stages of a plan3 on the operand slots (x0, x1, x2, ws).
static int run_plan3(const tnk_plan3* p, const double* x0, const double* x1, const double* x2,
                     double* out, double* ws, int64_t ws_elems, cudaStream_t st) {
    if (!p) {
        set_error("plan3: null plan");
        return TNK_ERR_ARG;
    }
    if (p->ws1_elems < 0 || p->ws2_elems < 0 || ws_elems < p->ws1_elems + p->ws2_elems) {
        set_error("plan3: workspace of %lld elements, plan needs %lld", (long long)ws_elems,
                  (long long)(p->ws1_elems + p->ws2_elems));
        return TNK_ERR_SIZE;
    }
    if (!out || (p->ws1_elems + p->ws2_elems > 0 && !ws)) {
        set_error("plan3: null output or workspace");
        return TNK_ERR_ARG;
    }
    Slots s{{x0, x1, x2, ws}};
    int rc = launch_gemm_f64(p->t1, p->s1, p->tiles1, p->n_tiles1, s, ws, st);
    if (rc) return rc;
    rc = launch_comb_f64(p->t2, p->c2, p->items2, p->n_items2, ws, ws, st);
    if (rc) return rc;
    rc = launch_gemm_f64(p->t3, p->s3, p->tiles3, p->n_tiles3, s, out, st);
    if (rc) return rc;
    return launch_comb_f64(p->t4, p->c4, p->items4, p->n_items4, ws, out, st);
}

}  // namespace tnk

using namespace tnk;

extern "C" {

const char* tnk_version(void) { return "tnkit_gb300 0.1.0 (sm_103a)"; }

const char* tnk_last_error(void) { return g_err; }

int tnk_struct_sizes(int64_t* out6) {
    if (!out6) return TNK_ERR_ARG;
    out6[0] = sizeof(tnk_gemm_task);
    out6[1] = sizeof(tnk_gemm_seg);
    out6[2] = sizeof(tnk_gemm_tile);
    out6[3] = sizeof(tnk_comb_task);
    out6[4] = sizeof(tnk_comb_term);
    out6[5] = sizeof(tnk_comb_item);
    return TNK_OK;
}

int tnk_contract3_f64(const tnk_plan3* plan, const double* x0, const double* x1,
                      const double* x2, double* out, double* ws, int64_t ws_elems,
                      void* stream) {
    return run_plan3(plan, x0, x1, x2, out, ws, ws_elems, (cudaStream_t)stream);
}

int tnk_apply_two_site_f64(const tnk_plan3* plan, const double* L, const double* theta,
                           const double* R, double* out, double* ws, int64_t ws_elems,
                           void* stream) {
    if (!L || !theta || !R) {
        set_error("apply_two_site: null operand");
        return TNK_ERR_ARG;
    }
    return run_plan3(plan, L, theta, R, out, ws, ws_elems, (cudaStream_t)stream);
}

int tnk_apply_one_site_f64(const tnk_plan3* plan, const double* L, const double* M,
                           const double* R, double* out, double* ws, int64_t ws_elems,
                           void* stream) {
    if (!L || !M || !R) {
        set_error("apply_one_site: null operand");
        return TNK_ERR_ARG;
    }
    return run_plan3(plan, L, M, R, out, ws, ws_elems, (cudaStream_t)stream);
}

int tnk_update_left_env_f64(const tnk_plan3* plan, const double* L, const double* A,
                            double* out, double* ws, int64_t ws_elems, void* stream) {
    if (!L || !A) {
        set_error("update_left_env: null operand");
        return TNK_ERR_ARG;
    }
    return run_plan3(plan, A, L, A, out, ws, ws_elems, (cudaStream_t)stream);
}

int tnk_update_right_env_f64(const tnk_plan3* plan, const double* R, const double* B,
                             double* out, double* ws, int64_t ws_elems, void* stream) {
    if (!R || !B) {
        set_error("update_right_env: null operand");
        return TNK_ERR_ARG;
    }
    return run_plan3(plan, B, R, B, out, ws, ws_elems, (cudaStream_t)stream);
}

int tnk_grouped_gemm_f64(const tnk_gemm_task* tasks, const tnk_gemm_seg* segs,
                         const tnk_gemm_tile* tiles, int64_t n_tiles, const double* b0,
                         const double* b1, const double* b2, const double* b3, double* C,
                         void* stream) {
    Slots s{{b0, b1, b2, b3}};
    return launch_gemm_f64(tasks, segs, tiles, n_tiles, s, C, (cudaStream_t)stream);
}

int tnk_combine_f64(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                    const tnk_comb_item* items, int64_t n_items, const double* src,
                    double* dst, void* stream) {
    return launch_comb_f64(tasks, terms, items, n_items, src, dst, (cudaStream_t)stream);
}

int tnk_dot_f64(const double* x, const double* y, int64_t n, double* out, double* red,
                void* stream) {
    if (!y) {
        set_error("dot: null y");
        return TNK_ERR_ARG;
    }
    return vec_dot(x, y, n, out, red, 0, (cudaStream_t)stream);
}

int tnk_nrm2_f64(const double* x, int64_t n, double* out, double* red, void* stream) {
    return vec_dot(x, nullptr, n, out, red, 1, (cudaStream_t)stream);
}

int tnk_multidot_f64(const double* V, int64_t ldv, int32_t nv, const double* w, int64_t n,
                     double* c, double* red, void* stream) {
    return vec_multidot(V, ldv, nv, w, n, c, red, (cudaStream_t)stream);
}

int tnk_gemv_sub_f64(const double* V, int64_t ldv, int32_t nv, const double* c, double* w,
                     int64_t n, void* stream) {
    return vec_gemv_sub(V, ldv, nv, c, w, n, (cudaStream_t)stream);
}

int tnk_cgs_pass_f64(const double* V, int64_t ldv, int32_t nv, const double* cin, double* w,
                     int64_t n, double* out, int32_t mode, double* red, uint32_t* counter,
                     void* stream) {
    return vec_cgs_pass(V, ldv, nv, cin, w, n, out, mode, red, counter, (cudaStream_t)stream);
}

int tnk_cgs_pass_seg_f64(const double* V, int64_t ldv, int32_t nv, const double* cin, double* w,
                         const int64_t* off, const int32_t* ids, int32_t nseg, int64_t max_len,
                         int64_t rec_stride, double* out, int32_t mode, double* red,
                         uint32_t* counter, void* stream) {
    return vec_cgs_pass_seg(V, ldv, nv, cin, w, off, ids, nseg, max_len, rec_stride, out, mode,
                            red, counter, (cudaStream_t)stream);
}

int tnk_scale_div_seg_f64(const double* x, double* y, const int64_t* off, const int32_t* ids,
                          int32_t nseg, int64_t max_len, const double* s, int64_t s_stride,
                          double f, void* stream) {
    return vec_scale_div_seg(x, y, off, ids, nseg, max_len, s, s_stride, f,
                             (cudaStream_t)stream);
}

int tnk_cgs_pass_f32(const float* V, int64_t ldv, int32_t nv, const double* cin, float* w,
                     int64_t n, double* out, int32_t mode, double* red, uint32_t* counter,
                     void* stream) {
    return vec_cgs_pass_f32(V, ldv, nv, cin, w, n, out, mode, red, counter,
                            (cudaStream_t)stream);
}

int tnk_scale_div_f32(const float* x, float* y, int64_t n, const double* s, double f,
                      void* stream) {
    return vec_scale_div_f32(x, y, n, s, f, (cudaStream_t)stream);
}

int tnk_rotate_f32(const float* V, int64_t ldv, int32_t nv, const double* Y, int32_t kk,
                   float* out, int64_t ldo, int64_t n, void* stream) {
    return vec_rotate_f32(V, ldv, nv, Y, kk, out, ldo, n, (cudaStream_t)stream);
}

int tnk_axpby_f64(const double* x, double* y, int64_t n, const double* sa, double fa,
                  const double* sb, double fb, void* stream) {
    return vec_axpby(x, y, n, sa, fa, sb, fb, (cudaStream_t)stream);
}

int tnk_scale_div_f64(const double* x, double* y, int64_t n, const double* s, double f,
                      void* stream) {
    return vec_scale_div(x, y, n, s, f, (cudaStream_t)stream);
}

}  // extern "C"
