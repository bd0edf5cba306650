// gch_fp32_pas.cu -- the passive-scalar stage kernels of the FP32-mixed policy
// (same flags as gch_fp32.cu).
#include "gch_engine.cuh"

namespace gch {
GCH_PASSIVE_FLUX(, PolMixed)
}
