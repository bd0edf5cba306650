// gch_tc32.cu -- thermal conduction on the FP32 paths (kernels in
// gch_tc.cuh), compiled like the other FP32 units.
#include "gch_tc.cuh"

namespace gch {

int tc_run_kahan(gch_domain* d, double dt_CFL) { return tc_run_t<PolKahan>(d, dt_CFL); }
int tc_run_mixed(gch_domain* d, double dt_CFL) { return tc_run_t<PolMixed>(d, dt_CFL); }

}  // namespace gch
