// gch_fp32.cu -- FP32-mixed instantiation of the timestep kernels (FP32
// fluxes, FP64 pressure recovery / accumulation / dt).  FMA contraction on.
#include "gch_engine.cuh"

namespace gch {
GCH_PASSIVE_FLUX(extern, PolMixed)
const EngineOps kEngineMixed = Engine<PolMixed>::ops();
}
