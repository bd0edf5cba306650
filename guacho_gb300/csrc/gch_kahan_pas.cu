// gch_kahan_pas.cu -- the passive-scalar stage kernels of the FP32 + Kahan policy
// (same flags as gch_kahan.cu).
#include "gch_engine.cuh"

namespace gch {
GCH_PASSIVE_FLUX(, PolKahan)
}
