// gch_fp64.cu -- FP64 (plain drop-in) instantiation of the timestep kernels.
// Built with -fmad=false: no FMA contraction, so every operation rounds like
// the reference's x86-64 FP64 build.
#include "gch_engine.cuh"

namespace gch {
GCH_PASSIVE_FLUX(extern, PolFP64)
const EngineOps kEngineFP64 = Engine<PolFP64>::ops();
}
