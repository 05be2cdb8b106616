// Pair-mode instantiations of the RHS + stage kernel: the FP64 body in FP32-pair arithmetic
// (ff.cuh), with the state, the RK accumulation and the state recovery in FP64.
#include "kernels_rhs.cuh"

namespace cns {
int launch_rhs_pair(int S, int V, const Geom& g, const Phys&, const CoefT<ff>& cf, const RhsIn<ff>& in,
                    const Update<ff>& up, double* scal, int quirk, cudaStream_t s) {
    return launch_rhs_t<ff>(S, V, g, cf, in, up, scal, quirk, s);
}
}  // namespace cns
