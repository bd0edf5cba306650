// gch_fp64_pas.cu -- the passive-scalar stage kernels of the FP64 policy (same
// flags as gch_fp64.cu).
#include "gch_engine.cuh"

namespace gch {
GCH_PASSIVE_FLUX(, PolFP64)
}
