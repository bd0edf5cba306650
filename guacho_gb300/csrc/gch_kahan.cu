// gch_kahan.cu -- FP32 + Kahan-compensated instantiation of the timestep
// kernels: u held as (hi, lo) FP32 pairs, no FP64 instruction on the per-cell
// path (FP64 runs at 1/57 of the FP32 rate on this part).
#include "gch_engine.cuh"

namespace gch {
GCH_PASSIVE_FLUX(extern, PolKahan)
const EngineOps kEngineKahan = Engine<PolKahan>::ops();
}
