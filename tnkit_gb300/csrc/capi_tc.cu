// extern "C" entry points of the tensor-core (mixed-precision) matvec.
#include "tnk_internal.cuh"

namespace tnk {
struct TcSeg;
struct CvtTask;
struct CvtItem;
int launch_gemm_tc(const tnk_gemm_task*, const TcSeg*, const tnk_gemm_tile*, int64_t,
                   const void*, void*, int*, int, int, cudaStream_t, bool);
int encode_tmaps(const float*, const int64_t*, int64_t, void*, int);
int launch_cvt_split(const CvtTask*, const CvtItem*, int64_t, const double*, float*, int64_t,
                     int, cudaStream_t);
int launch_comb_f32(const tnk_comb_task*, const tnk_comb_term*, const tnk_comb_item*, int64_t,
                    const float*, float*, int64_t, int, cudaStream_t, bool);
}  // namespace tnk

using namespace tnk;

extern "C" {

int tnk_stage_f32(const tnk_cvt_task* tasks, const tnk_cvt_item* items, int64_t n_items,
                  const double* src, float* dst, int64_t lo_off, int32_t split, void* stream) {
    return launch_cvt_split(reinterpret_cast<const CvtTask*>(tasks),
                            reinterpret_cast<const CvtItem*>(items), n_items, src, dst, lo_off,
                            split, (cudaStream_t)stream);
}

int tnk_tc_encode_tmaps(const float* base, const int64_t* desc4, int64_t n, void* out) {
    if (!base || !desc4 || !out || n < 0) {
        set_error("encode tensor maps: bad argument");
        return TNK_ERR_ARG;
    }
    return encode_tmaps(base, desc4, n, out, 4);
}

int tnk_tc_encode_tmaps_box(const float* base, const int64_t* desc5, int64_t n, void* out) {
    if (!base || !desc5 || !out || n < 0) {
        set_error("encode tensor maps: bad argument");
        return TNK_ERR_ARG;
    }
    return encode_tmaps(base, desc5, n, out, 5);
}

int tnk_grouped_gemm_tc(const tnk_gemm_task* tasks, const tnk_tc_seg* segs,
                        const tnk_gemm_tile* tiles, int64_t n_tiles, const void* maps, void* C,
                        int* err, int32_t passes, void* stream) {
    return launch_gemm_tc(tasks, reinterpret_cast<const TcSeg*>(segs), tiles, n_tiles, maps, C,
                          err, passes, 128, (cudaStream_t)stream, false);
}

int tnk_grouped_gemm_tc_bn(const tnk_gemm_task* tasks, const tnk_tc_seg* segs,
                           const tnk_gemm_tile* tiles, int64_t n_tiles, const void* maps,
                           void* C, int* err, int32_t passes, int32_t bn, void* stream) {
    return launch_gemm_tc(tasks, reinterpret_cast<const TcSeg*>(segs), tiles, n_tiles, maps, C,
                          err, passes, bn, (cudaStream_t)stream, false);
}

int tnk_combine_f32(const tnk_comb_task* tasks, const tnk_comb_term* terms,
                    const tnk_comb_item* items, int64_t n_items, const float* src, float* dst,
                    int64_t lo_off, int32_t split, void* stream) {
    return launch_comb_f32(tasks, terms, items, n_items, src, dst, lo_off, split,
                           (cudaStream_t)stream, false);
}

int tnk_apply_two_site_tc(const tnk_tc_plan* p, const double* theta, double* out,
                          void* stream) {
    if (!p || !theta || !out || !p->stage || !p->y32 || !p->err || !p->maps) {
        set_error("apply_two_site_tc: null plan, buffer or operand");
        return TNK_ERR_ARG;
    }
    const int split = p->passes == 3;
    const int bn3 = p->bn3 == 0 ? 128 : p->bn3;
    if (bn3 != 128 && bn3 != 64) {
        set_error("apply_two_site_tc: stage-3 tile width %d (128 or 64)", p->bn3);
        return TNK_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // theta's staging waits for everything before it on the stream; the three kernels after it
    // are programmatic dependents of their predecessor, so each one's launch and prologue (TMEM
    // allocation, barrier set-up, plan reads) overlap the previous kernel's tail
    int rc = launch_cvt_split(reinterpret_cast<const CvtTask*>(p->cvt),
                              reinterpret_cast<const CvtItem*>(p->cvt_items), p->n_cvt_items,
                              theta, p->stage, p->lo_off, split, st);
    if (rc) return rc;
    rc = launch_gemm_tc(p->t1, reinterpret_cast<const TcSeg*>(p->s1), p->tiles1, p->n_tiles1,
                        p->maps, p->y32, p->err, p->passes, 128, st, true);
    if (rc) return rc;
    rc = launch_comb_f32(p->t2, p->c2, p->items2, p->n_items2, p->y32, p->stage, p->lo_off,
                         split, st, true);
    if (rc) return rc;
    return launch_gemm_tc(p->t3, reinterpret_cast<const TcSeg*>(p->s3), p->tiles3, p->n_tiles3,
                          p->maps, out, p->err, p->passes, bn3, st, true);
}

}  // extern "C"
