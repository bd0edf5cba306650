// gch_kahan_grp.cu -- grouped many-box kernels, FP32 + Kahan-pair policy
// (compiled apart from gch_kahan.cu so the two build in parallel).
#include "gch_group_engine.cuh"

namespace gch {
const GroupOps kGroupKahan = GroupEngine<PolKahan>::ops();
}
