// Variant registry of the 2D ensemble stage kernel.
#include "sc_ens.cuh"
namespace sc {
EnsVariant ens_variant_f32_v0();
EnsVariant ens_variant_f32_v1();
EnsVariant ens_variant_f32_v2();
EnsVariant ens_variant_f32_v3();
EnsVariant ens_variant_f32_v4();
EnsVariant ens_variant_f32_v5();
EnsVariant ens_variant_f64_v0();
EnsVariant ens_variant_f64_v1();

EnsVariant ens_variant_f32(int v) {
  switch (v) {
    case 0: return ens_variant_f32_v0();
    case 1: return ens_variant_f32_v1();
    case 2: return ens_variant_f32_v2();
    case 3: return ens_variant_f32_v3();
    case 4: return ens_variant_f32_v4();
    case 5: return ens_variant_f32_v5();
    default: return EnsVariant{nullptr, 0, 0, 0, 0, 0, 0};
  }
}

EnsVariant ens_variant_f64(int v) {
  switch (v) {
    case 0: return ens_variant_f64_v0();
    case 1: return ens_variant_f64_v1();
    default: return EnsVariant{nullptr, 0, 0, 0, 0, 0, 0};
  }
}
}  // namespace sc
