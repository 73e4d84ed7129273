// Compiled instance: 2D ensemble stage kernel, double, variant 0 (EnsShape<256, 2, 4096, 8, false>).
#include "sc_ens.cuh"
namespace sc {
EnsVariant ens_variant_f64_v0() { return ens_variant_of<EnsShape<256, 2, 4096, 8, false>, double>(); }
}  // namespace sc
