// gch_fp32_grp.cu -- grouped many-box kernels, FP32-mixed policy (compiled
// apart from gch_fp32.cu so the two build in parallel).
#include "gch_group_engine.cuh"

namespace gch {
const GroupOps kGroupMixed = GroupEngine<PolMixed>::ops();
}
