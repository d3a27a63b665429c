// Run-time selection among the compiled step kernel variants (step_inst.cu objects).
#include "launch.h"

namespace lbffs {

#define LBFFS_DECL4(Q, S, C)                                                          \
    cudaError_t launch_step_q##Q##_s##S##_c##C##_p0(const StepArgs&, cudaStream_t); \
    cudaError_t launch_step_q##Q##_s##S##_c##C##_p1(const StepArgs&, cudaStream_t); \
    cudaError_t launch_step_q##Q##_s##S##_c##C##_p2(const StepArgs&, cudaStream_t); \
    cudaError_t launch_step_q##Q##_s##S##_c##C##_p3(const StepArgs&, cudaStream_t);
LBFFS_DECL4(19, 0, 0)
LBFFS_DECL4(19, 1, 0)
LBFFS_DECL4(19, 2, 0)
LBFFS_DECL4(27, 0, 0)
LBFFS_DECL4(27, 1, 0)
LBFFS_DECL4(27, 2, 0)
LBFFS_DECL4(27, 0, 1)
LBFFS_DECL4(27, 1, 1)
LBFFS_DECL4(27, 2, 1)
#undef LBFFS_DECL4

typedef cudaError_t (*StepFn)(const StepArgs&, cudaStream_t);

#define LBFFS_ROW(Q, S, C)                                                                                   \
    {                                                                                                        \
        launch_step_q##Q##_s##S##_c##C##_p0, launch_step_q##Q##_s##S##_c##C##_p1,                            \
            launch_step_q##Q##_s##S##_c##C##_p2, launch_step_q##Q##_s##S##_c##C##_p3                         \
    }

// [storage][part]
static const StepFn k19[3][4] = {LBFFS_ROW(19, 0, 0), LBFFS_ROW(19, 1, 0), LBFFS_ROW(19, 2, 0)};
// [collision][storage][part]
static const StepFn k27[2][3][4] = {{LBFFS_ROW(27, 0, 0), LBFFS_ROW(27, 1, 0), LBFFS_ROW(27, 2, 0)},
                                    {LBFFS_ROW(27, 0, 1), LBFFS_ROW(27, 1, 1), LBFFS_ROW(27, 2, 1)}};
#undef LBFFS_ROW

static int part_of(const StepConfig& c, bool bulk)
{
    if (!bulk) return 3;
    if (c.sgs == SGS_WALE) return 2;
    return c.les ? 1 : 0;
}

cudaError_t launch_q19(const StepArgs& a, const StepConfig& c, bool bulk, cudaStream_t st)
{
    if (c.storage < 0 || c.storage > 2) return cudaErrorInvalidValue;
    if (bulk && a.bulk_kind == 1) {
        const bool les = c.sgs != SGS_WALE && c.les;
        if (c.storage == ST_FP32) return launch_bulk_tma_s0(a, c.sgs, les, st);
        if (c.storage == ST_FP16S) return launch_bulk_tma_s1(a, c.sgs, les, st);
        return launch_bulk_tma_s2(a, c.sgs, les, st);
    }
    return k19[c.storage][part_of(c, bulk)](a, st);
}

cudaError_t launch_q27(const StepArgs& a, const StepConfig& c, bool bulk, cudaStream_t st)
{
    if (c.storage < 0 || c.storage > 2 || c.collision < 0 || c.collision > 1) return cudaErrorInvalidValue;
    return k27[c.collision][c.storage][part_of(c, bulk)](a, st);
}

}  // namespace lbffs
