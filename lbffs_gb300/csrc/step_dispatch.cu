// Run-time selection among the compiled step kernel variants (step_inst.cu objects).
#include "launch.h"

namespace lbffs {

#define LBFFS_DECL(Q, S)                                                                                 \
    cudaError_t launch_bulk_q##Q##_s##S##_inst(const StepArgs&, const StepConfig&, cudaStream_t);      \
    cudaError_t launch_special_q##Q##_s##S##_inst(const StepArgs&, const StepConfig&, cudaStream_t);
LBFFS_DECL(19, 0)
LBFFS_DECL(19, 1)
LBFFS_DECL(19, 2)
LBFFS_DECL(27, 0)
LBFFS_DECL(27, 1)
LBFFS_DECL(27, 2)
#undef LBFFS_DECL

#define LBFFS_PICK(Q)                                                                                    \
    switch (c.storage) {                                                                                 \
        case ST_FP32: return bulk ? launch_bulk_q##Q##_s0_inst(a, c, st) : launch_special_q##Q##_s0_inst(a, c, st); \
        case ST_FP16S: return bulk ? launch_bulk_q##Q##_s1_inst(a, c, st) : launch_special_q##Q##_s1_inst(a, c, st); \
        case ST_BF16S: return bulk ? launch_bulk_q##Q##_s2_inst(a, c, st) : launch_special_q##Q##_s2_inst(a, c, st); \
    }                                                                                                    \
    return cudaErrorInvalidValue;

cudaError_t launch_q19(const StepArgs& a, const StepConfig& c, bool bulk, cudaStream_t st) { LBFFS_PICK(19) }
cudaError_t launch_q27(const StepArgs& a, const StepConfig& c, bool bulk, cudaStream_t st) { LBFFS_PICK(27) }

}  // namespace lbffs
