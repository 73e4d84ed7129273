// Compiled instance: 2D ensemble stage kernel, float, variant 4 (EnsShape<256, 2, 4096, 4, false>).
#include "sc_ens.cuh"
namespace sc {
EnsVariant ens_variant_f32_v4() { return ens_variant_of<EnsShape<256, 2, 4096, 4, false>, float>(); }
}  // namespace sc
