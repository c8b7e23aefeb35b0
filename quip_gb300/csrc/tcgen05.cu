// tcgen05.cu -- K5 mixed path (placeholder until the tensor-core GEMMs land).
#include "context.h"

namespace gapgpu {

int prepare_mixed_operands(gapgpu_model&) { return GAPGPU_OK; }

int gp_mixed(gapgpu_context&, const Coordinate&, int, int) {
    GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "mixed-precision GEMMs are not built yet");
}

}  // namespace gapgpu
