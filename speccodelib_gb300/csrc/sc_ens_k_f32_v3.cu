// Compiled instance: 2D ensemble stage kernel, float, variant 3 (EnsShape<512, 1, 8192, 8, true>).
#include "sc_ens.cuh"
namespace sc {
EnsVariant ens_variant_f32_v3() { return ens_variant_of<EnsShape<512, 1, 8192, 8, true>, float>(); }
}  // namespace sc
