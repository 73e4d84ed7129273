// Compiled instance: 2D ensemble stage kernel, float, variant 1 (EnsShape<256, 2, 4096, 8, true>).
#include "sc_ens.cuh"
namespace sc {
EnsVariant ens_variant_f32_v1() { return ens_variant_of<EnsShape<256, 2, 4096, 8, true>, float>(); }
}  // namespace sc
