// Compiled instance: 2D ensemble stage kernel, float, variant 2 (EnsShape<512, 1, 8192, 8, false>).
#include "sc_ens.cuh"
namespace sc {
EnsVariant ens_variant_f32_v2() { return ens_variant_of<EnsShape<512, 1, 8192, 8, false>, float>(); }
}  // namespace sc
