// FP64 instantiations of the RHS + stage kernel (plain path).
#include "kernels_rhs.cuh"

namespace cns {
int launch_rhs_fp64(int S, int V, const Geom& g, const Phys&, const CoefT<double>& cf, const RhsIn<double>& in,
                    const Update<double>& up, double* scal, int quirk, cudaStream_t s) {
    return launch_rhs_t<double>(S, V, g, cf, in, up, scal, quirk, s);
}
}  // namespace cns
