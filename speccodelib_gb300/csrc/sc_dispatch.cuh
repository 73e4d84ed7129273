// Runtime-length dispatch of the pass kernels (compiled per precision and per
// kernel family in separate translation units so the build runs in parallel).
#pragma once
#include "sc_launch.h"
#include "sc_ops.cuh"
#include "sc_tma_passes.cuh"
#include "sc_xwarp.cuh"
#include "sc_adjoint.cuh"
#include "sc_fused.cuh"

namespace sc {

// Raise the dynamic shared-memory limit once per kernel instance.
template <typename K> inline cudaError_t smem_attr(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

#define SC_LOGN_CASES(X) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10)
#define SC_LOGM_CASES(X) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9)

template <typename T, int LOGN, bool INV>
cudaError_t launch_plain(const FieldList<T>& fl, const PlainArgs<T>& pa, const Geom& g, int nouter,
                         const C2<T>* tw, cudaStream_t s) {
  using Cfg = PencilCfg<T, LOGN>;
  auto k = pencil_plain_kernel<T, LOGN, INV>;
  static cudaError_t attr = smem_attr(k, Cfg::SMEM);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Cfg::P - 1) / Cfg::P, nouter);
  k<<<grid, Cfg::NT, Cfg::SMEM, s>>>(fl, pa, g, tw);
  return cudaGetLastError();
}

template <typename T, int LOGN, int MODE>
cudaError_t launch_zinv(const ZvArgs<T>& za, const FieldList<T>& out, const Geom& g,
                        const C2<T>* tw, cudaStream_t s) {
  using Cfg = PencilCfg<T, LOGN>;
  auto k = zinv_vel_kernel<T, LOGN, MODE>;
  static cudaError_t attr = smem_attr(k, Cfg::SMEM);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Cfg::P - 1) / Cfg::P, g.ny);
  if (za.tiles_x > 0 && (unsigned)za.tiles_x < grid.x) grid.x = za.tiles_x;
  k<<<grid, Cfg::NT, Cfg::SMEM, s>>>(za, out, g, tw);
  return cudaGetLastError();
}

template <typename T, int LOGN, int NIN>
cudaError_t launch_zfwd(const FieldList<T>& fin, const StageArgs<T>& st, const Geom& g,
                        const C2<T>* tw, cudaStream_t s) {
  using Cfg = PencilCfg<T, LOGN>;
  auto k = zfwd_stage_kernel<T, LOGN, NIN>;
  static cudaError_t attr = smem_attr(k, Cfg::SMEM);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Cfg::P - 1) / Cfg::P, g.ny);
  k<<<grid, Cfg::NT, Cfg::SMEM, s>>>(fin, st, g, tw);
  return cudaGetLastError();
}

template <typename T, int LOGM, int MODE>
cudaError_t launch_xpass(const FieldList<T>& fin, const FieldList<T>& fout, const Geom& g,
                         const C2<T>* twM, const C2<T>* twN, const XArgs<T>& xa, cudaStream_t s) {
  using Cfg = XpCfg<T, LOGM, MODE>;
  auto k = xpass_kernel<T, LOGM, MODE>;
  static cudaError_t attr = smem_attr(k, Cfg::SMEM);
  if (attr != cudaSuccess) return attr;
  const long long nb = (xa.rows + Cfg::RB - 1) / Cfg::RB;
  k<<<(unsigned)nb, Cfg::NT, Cfg::SMEM, s>>>(fin, fout, g, twM, twN, xa);
  return cudaGetLastError();
}

template <typename T, int LOGN, bool INV>
cudaError_t launch_plain_tma(const CUtensorMap& map, const TmaPass<T>& tp, const Geom& g, const C2<T>* tw,
                             int nsm, cudaStream_t s) {
  using Cfg = TmaCfg<T, LOGN>;
  auto k = pencil_tma_kernel<T, LOGN, INV>;
  constexpr size_t sm = Cfg::STAGES * Cfg::TILE_BYTES + kSmemAlignPad;
  static cudaError_t attr = smem_attr(k, sm);
  if (attr != cudaSuccess) return attr;
  const long long total = (long long)tp.ntx * tp.nouter * tp.nf;
  long long grid = (long long)nsm * 2;
  if (grid > total) grid = total;
  k<<<(unsigned)grid, Cfg::NT, sm, s>>>(map, tp, g, tw);
  return cudaGetLastError();
}

template <typename T, int LOGN>
cudaError_t launch_zinv_tma(const CUtensorMap& vmap, const ZvArgs<T>& za, const FieldList<T>& out,
                            const Geom& g, const C2<T>* tw, int* err, cudaStream_t s) {
  using Cfg = TmaCfg<T, LOGN>;
  auto k = zinv_tma_kernel<T, LOGN>;
  constexpr size_t sm = 3 * Cfg::TILEZ_BYTES + Cfg::WORKZ_BYTES + kSmemAlignPad;
  static cudaError_t attr = smem_attr(k, sm);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Cfg::PZ - 1) / Cfg::PZ, g.ny);
  k<<<grid, Cfg::NTZ, sm, s>>>(vmap, za, out, g, tw, err);
  return cudaGetLastError();
}

template <typename T, int LOGN, int NIN>
cudaError_t launch_zfwd_fields_tma(const CUtensorMap& fmap, const StageArgs<T>& st, const Geom& g, const C2<T>* tw,
                                   int* err, cudaStream_t s) {
  using Cfg = TmaCfg<T, LOGN>;
  auto k = zfwd_fields_tma_kernel<T, LOGN, NIN>;
  constexpr size_t sm = 3 * Cfg::TILE_BYTES + kSmemAlignPad;
  static cudaError_t attr = smem_attr(k, sm);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Cfg::P - 1) / Cfg::P, g.ny);
  k<<<grid, Cfg::NT, sm, s>>>(fmap, st, g, tw, err);
  return cudaGetLastError();
}

template <typename T, int LOGN, int MODE>
cudaError_t launch_zfwd_tma_mode(const CUtensorMap& lmap, const CUtensorMap& vmap, int vstore, const StageArgs<T>& st,
                                 const Geom& g, const C2<T>* tw, int* err, cudaStream_t s) {
  using Cfg = TmaCfg<T, LOGN>;
  auto k = zfwd_tma_kernel<T, LOGN, MODE>;
  constexpr size_t sm = 3 * Cfg::TILE_BYTES + kSmemAlignPad;
  static cudaError_t attr = smem_attr(k, sm);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Cfg::P - 1) / Cfg::P, g.ny);
  k<<<grid, ZfCfg<T, LOGN>::NT, sm, s>>>(lmap, vmap, vstore, st, g, tw, err);
  return cudaGetLastError();
}

// RK stage 4 (the step's last) in its own instance, the state stored from the
// tiles when vstore; other modes read st.mode at run time
template <typename T, int LOGN>
cudaError_t launch_zfwd_tma(const CUtensorMap& lmap, const CUtensorMap& vmap, int vstore, const StageArgs<T>& st,
                            const Geom& g, const C2<T>* tw, int* err, cudaStream_t s) {
  if (st.mode == SM_RK4) return launch_zfwd_tma_mode<T, LOGN, SM_RK4>(lmap, vmap, vstore, st, g, tw, err, s);
  // the variable-step AB2 with its update in the epilogue has an instance of its own
  if (st.mode == SM_AB2V) return launch_zfwd_tma_mode<T, LOGN, SM_AB2V>(lmap, vmap, 0, st, g, tw, err, s);
  return launch_zfwd_tma_mode<T, LOGN, -1>(lmap, vmap, 0, st, g, tw, err, s);
}

template <typename T, int LOGN, int MODE>
cudaError_t launch_zfwd_zinv_mode(const CUtensorMap& lmap, const CUtensorMap& fmap, const StageArgs<T>& st,
                                  const FusedArgs<T>& fa, const Geom& g, const C2<T>* tw, int* err,
                                  cudaStream_t s) {
  using Z = ZiCfg<T, LOGN>;
  auto k = zfwd_zinv_tma_kernel<T, LOGN, MODE>;
  static cudaError_t attr = smem_attr(k, Z::SMEM);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Z::P - 1) / Z::P, g.ny);
  k<<<grid, Z::NT, Z::SMEM, s>>>(lmap, fmap, st, fa, g, tw, err);
  return cudaGetLastError();
}

// one instance per RK stage (the update's mode a compile-time constant;
// SC_FUSED_RUNTIME_MODE: one instance reading it at run time)
template <typename T, int LOGN>
cudaError_t launch_zfwd_zinv(const CUtensorMap& lmap, const CUtensorMap& fmap, const StageArgs<T>& st,
                             const FusedArgs<T>& fa, const Geom& g, const C2<T>* tw, int* err, cudaStream_t s) {
  using Z = ZiCfg<T, LOGN>;
  if constexpr (!Z::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
#ifdef SC_FUSED_RUNTIME_MODE
    return launch_zfwd_zinv_mode<T, LOGN, -1>(lmap, fmap, st, fa, g, tw, err, s);
#else
    switch (st.mode) {
      case SM_RK1: return launch_zfwd_zinv_mode<T, LOGN, SM_RK1>(lmap, fmap, st, fa, g, tw, err, s);
      case SM_RK2: return launch_zfwd_zinv_mode<T, LOGN, SM_RK2>(lmap, fmap, st, fa, g, tw, err, s);
      case SM_RK3: return launch_zfwd_zinv_mode<T, LOGN, SM_RK3>(lmap, fmap, st, fa, g, tw, err, s);
      default: return cudaErrorNotSupported;
    }
#endif
  }
}

template <typename T, int LOGN>
cudaError_t launch_zinv_phi(const CUtensorMap& lmap, const CUtensorMap& omap, const ZvArgs<T>& za,
                            const FieldList<T>& out, const Geom& g, const C2<T>* tw, int* err, cudaStream_t s) {
  using Z = ZiCfg<T, LOGN>;
  if constexpr (!Z::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    auto k = zinv_phi_tma_kernel<T, LOGN>;
    static cudaError_t attr = smem_attr(k, Z::SMEM);
    if (attr != cudaSuccess) return attr;
    dim3 grid((g.nxh + Z::P - 1) / Z::P, g.ny);
    k<<<grid, Z::NT, Z::SMEM, s>>>(lmap, omap, za, out, g, tw, err);
    return cudaGetLastError();
  }
}

template <typename T, int LOGN, int MODE>
cudaError_t launch_zinv5(const CUtensorMap& vmap, const CUtensorMap& umap, const ZvArgs<T>& za,
                         const FieldList<T>& out, const Geom& g, const C2<T>* tw, int* err, cudaStream_t s) {
  using Z = ZiCfg<T, LOGN>;
  if constexpr (!Z::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    auto k = zinv5_tma_kernel<T, LOGN, MODE>;
    static cudaError_t attr = smem_attr(k, Z::SMEM);
    if (attr != cudaSuccess) return attr;
    dim3 grid((g.nxh + Z::P - 1) / Z::P, g.ny);
    if (za.tiles_x > 0 && (unsigned)za.tiles_x < grid.x) grid.x = za.tiles_x;
    k<<<grid, Z::NT, Z::SMEM, s>>>(vmap, umap, za, out, g, tw, err);
    return cudaGetLastError();
  }
}

template <typename T, int LOGM, int MODE>
cudaError_t launch_xwarp(const FieldList<T>& fin, const FieldList<T>& fout, const Geom& g, const C2<T>* twM,
                         const C2<T>* twN, const XArgs<T>& xa, cudaStream_t s) {
  using Cfg = XwCfg<T, LOGM, MODE>;
  auto k = xpass_warp_kernel<T, LOGM, MODE>;
  static cudaError_t attr = smem_attr(k, Cfg::SMEM_LAUNCH);
  if (attr != cudaSuccess) return attr;
  const long long nb = (xa.rows + Cfg::WARPS - 1) / Cfg::WARPS;
  k<<<(unsigned)nb, Cfg::NT, Cfg::SMEM_LAUNCH, s>>>(fin, fout, g, twM, twN, xa);
  return cudaGetLastError();
}

template <typename T, int LOGN>
cudaError_t launch_zfwd_adj(const FieldList<T>& fin, const AdjArgs<T>& aa, const Geom& g, const C2<T>* tw,
                            cudaStream_t s) {
  using Cfg = PencilCfg<T, LOGN>;
  auto k = zfwd_adj_kernel<T, LOGN>;
  static cudaError_t attr = smem_attr(k, Cfg::SMEM);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + Cfg::P - 1) / Cfg::P, g.ny);
  k<<<grid, Cfg::NT, Cfg::SMEM, s>>>(fin, aa, g, tw);
  return cudaGetLastError();
}

template <typename T, int LOGN>
cudaError_t launch_zfwd_adj_tma(const CUtensorMap& pmap, const int fidx[6], const AdjArgs<T>& aa, const Geom& g,
                                const C2<T>* tw, int* err, cudaStream_t s) {
  using AC = AdjTmaCfg<T, LOGN>;
  auto k = zfwd_adj_tma_kernel<T, LOGN>;
  static cudaError_t attr = smem_attr(k, AC::SMEM);
  if (attr != cudaSuccess) return attr;
  dim3 grid((g.nxh + AC::P - 1) / AC::P, g.ny);
  const int4 lo = make_int4(fidx[0], fidx[1], fidx[2], fidx[3]);
  const int2 hi = make_int2(fidx[4], fidx[5]);
  k<<<grid, AC::NT, AC::SMEM, s>>>(pmap, lo, hi, aa, g, tw, err);
  return cudaGetLastError();
}

}  // namespace sc

#define SC_ZFWDADJTMA_CASE(L) case L: return sc::launch_zfwd_adj_tma<ADJ_T, L>(pmap, fidx, aa, g, tw, err, s);
#define SC_ADJTILE_CASE(L) case L: return sc::AdjTmaCfg<ADJ_T, L>::P;
#define SC_ZFWDADJ_CASE(L) case L: return sc::launch_zfwd_adj<ADJ_T, L>(fin, aa, g, tw, s);
#define SC_DEFINE_ADJ(T)                                                                         \
  template <> int sc::Launch<T>::adj_tile(int logn) {                                            \
    switch (logn) { SC_LOGN_CASES(SC_ADJTILE_CASE) default: return 0; }                           \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zfwd_adj_tma(int logn, const CUtensorMap& pmap, const int fidx[6],  \
                                          const AdjArgs<T>& aa, const Geom& g, const C2<T>* tw,  \
                                          int* err, cudaStream_t s) {                            \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZFWDADJTMA_CASE)                                                          \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zfwd_adj(int logn, const FieldList<T>& fin, const AdjArgs<T>& aa,   \
                                      const Geom& g, const C2<T>* tw, cudaStream_t s) {          \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZFWDADJ_CASE)                                                             \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::adj_copyT(const FieldList<T>& lw, const Geom& g, cudaStream_t s) {  \
    long long n = (long long)g.ny * g.nz;                                                        \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 4096) nb = 4096;                                                                    \
    sc::adj_copyT_kernel<T><<<nb, 256, 0, s>>>(lw, g);                                           \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::adj_op(const AdjOpArgs<T>& ao, const Geom& g, cudaStream_t s) {     \
    long long n = (long long)g.ny * g.nz * g.nxh;                                                \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 152 * 16) nb = 152 * 16;                                                            \
    sc::adj_op_kernel<T><<<nb, 256, 0, s>>>(ao, g);                                              \
    return cudaGetLastError();                                                                   \
  }

#define SC_DEFINE_XWARP(T, CASES)                                                                \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::xpass_warp(int logm, int mode, const FieldList<T>& fin,             \
                                        const FieldList<T>& fout, const Geom& g,                 \
                                        const C2<T>* twM, const C2<T>* twN,                      \
                                        const XArgs<T>& xa, cudaStream_t s) {                    \
    switch (logm) {                                                                              \
      CASES                                                                                      \
      default: return cudaErrorNotSupported;                                                     \
    }                                                                                            \
  }

#define SC_XWARP_CASE(T, L)                                                                      \
  case L:                                                                                        \
    return mode == sc::XW_ADJ    ? sc::launch_xwarp<T, L, sc::XW_ADJ>(fin, fout, g, twM, twN, xa, s)  \
           : mode == sc::XW_SMAG ? sc::launch_xwarp<T, L, sc::XW_SMAG>(fin, fout, g, twM, twN, xa, s) \
                                 : sc::launch_xwarp<T, L, sc::XW_DNS>(fin, fout, g, twM, twN, xa, s);

#define SC_TMA_TILE_CASE(L) case L: return sc::TmaCfg<TMA_T, L>::P;
#define SC_TMA_ZTILE_CASE(L) case L: return sc::TmaCfg<TMA_T, L>::PZ;

#define SC_DEFINE_TMA(T)                                                                         \
  template <> int sc::Launch<T>::tma_tile(int logn) {                                            \
    switch (logn) { SC_LOGN_CASES(SC_TMA_TILE_CASE) default: return 0; }                         \
  }                                                                                              \
  template <> int sc::Launch<T>::tma_ztile(int logn) {                                           \
    switch (logn) { SC_LOGN_CASES(SC_TMA_ZTILE_CASE) default: return 0; }                        \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::plain_tma(int logn, bool inv, const CUtensorMap& map,               \
                                       const TmaPass<T>& tp, const Geom& g, const C2<T>* tw,     \
                                       int nsm, cudaStream_t s) {                                \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_PLAINTMA_CASE_##T)                                                        \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zinv_tma(int logn, const CUtensorMap& vmap, const ZvArgs<T>& za,    \
                                      const FieldList<T>& out, const Geom& g, const C2<T>* tw,   \
                                      int* err, cudaStream_t s) {                                \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZINVTMA_CASE_##T)                                                         \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zfwd_fields_tma(int logn, int nin, const CUtensorMap& fmap,         \
                                             const StageArgs<T>& st, const Geom& g,              \
                                             const C2<T>* tw, int* err, cudaStream_t s) {        \
    if (nin != 9) return cudaErrorNotSupported;                                                  \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZFWDFIELDS_CASE_##T)                                                      \
      default: return cudaErrorNotSupported;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zfwd_tma(int logn, const CUtensorMap& lmap, const CUtensorMap& vmap,  \
                                      int vstore, const StageArgs<T>& st, const Geom& g,         \
                                      const C2<T>* tw, int* err, cudaStream_t s) {               \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZFWDTMA_CASE_##T)                                                         \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }

#define SC_PLAINTMA_CASE_float(L) \
  case L: return inv ? sc::launch_plain_tma<float, L, true>(map, tp, g, tw, nsm, s) \
                     : sc::launch_plain_tma<float, L, false>(map, tp, g, tw, nsm, s);
#define SC_PLAINTMA_CASE_double(L) \
  case L: return inv ? sc::launch_plain_tma<double, L, true>(map, tp, g, tw, nsm, s) \
                     : sc::launch_plain_tma<double, L, false>(map, tp, g, tw, nsm, s);
#define SC_ZINVTMA_CASE_float(L) case L: return sc::launch_zinv_tma<float, L>(vmap, za, out, g, tw, err, s);
#define SC_ZINVTMA_CASE_double(L) case L: return sc::launch_zinv_tma<double, L>(vmap, za, out, g, tw, err, s);
#define SC_ZFWDFIELDS_CASE_float(L) case L: return sc::launch_zfwd_fields_tma<float, L, 9>(fmap, st, g, tw, err, s);
#define SC_ZFWDFIELDS_CASE_double(L) case L: return sc::launch_zfwd_fields_tma<double, L, 9>(fmap, st, g, tw, err, s);
#define SC_ZFWDTMA_CASE_float(L) case L: return sc::launch_zfwd_tma<float, L>(lmap, vmap, vstore, st, g, tw, err, s);
#define SC_ZFWDTMA_CASE_double(L) case L: return sc::launch_zfwd_tma<double, L>(lmap, vmap, vstore, st, g, tw, err, s);

#define SC_DEFINE_TILE(T) \
  template <> int sc::Launch<T>::tile() { return sc::Tile<T>::P; }

#define SC_DEFINE_PLAIN(T)                                                                       \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::plain(int logn, bool inv, const FieldList<T>& fl,                   \
                                   const PlainArgs<T>& pa, const Geom& g, int nouter,            \
                                   const C2<T>* tw, cudaStream_t s) {                            \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_PLAIN_CASE_##T)                                                           \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }

#define SC_DEFINE_ZINV(T)                                                                        \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zinv_vel(int logn, int mode, const ZvArgs<T>& za,                   \
                                      const FieldList<T>& out, const Geom& g, const C2<T>* tw,   \
                                      cudaStream_t s) {                                          \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZINV_CASE_##T)                                                            \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }

#define SC_DEFINE_ZFWD(T)                                                                        \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zfwd_stage(int logn, int nin, const FieldList<T>& fin,              \
                                        const StageArgs<T>& st, const Geom& g, const C2<T>* tw,  \
                                        cudaStream_t s) {                                        \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZFWD_CASE_##T)                                                            \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::fixup(const StageArgs<T>& st, const Geom& g, cudaStream_t s) {      \
    long long n = (long long)g.ny * g.nz;                                                        \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 4096) nb = 4096;                                                                    \
    if (st.mode == sc::SM_AB2V) sc::fixup_kx0_kernel<T, sc::SM_AB2V><<<nb, 256, 0, s>>>(st, g);   \
    else sc::fixup_kx0_kernel<T><<<nb, 256, 0, s>>>(st, g);                                      \
    return cudaGetLastError();                                                                   \
  }

#define SC_DEFINE_XPASS(T)                                                                       \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::xpass(int logm, int mode, const FieldList<T>& fin,                  \
                                   const FieldList<T>& fout, const Geom& g, const C2<T>* twM,    \
                                   const C2<T>* twN, const XArgs<T>& xa, cudaStream_t s) {       \
    switch (logm) {                                                                              \
      SC_LOGM_CASES(SC_XPASS_CASE_##T)                                                           \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }

#define SC_DEFINE_OPS(T)                                                                         \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::diag(const DiagArgs<T>& da, const Geom& g, cudaStream_t s) {        \
    size_t sm = sizeof(double) * (size_t)da.nshell;                                              \
    sc::diag_partial_kernel<T><<<da.nblocks, 256, sm, s>>>(da, g);                               \
    cudaError_t e = cudaGetLastError();                                                          \
    if (e != cudaSuccess) return e;                                                              \
    sc::diag_final_kernel<<<1, 256, 0, s>>>(da.partial, da.nblocks, sc::DQ_N + da.nshell,        \
                                            da.out);                                             \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::specop(const SpecOpArgs<T>& oa, const Geom& g, cudaStream_t s) {    \
    long long n = (long long)g.ny * g.nz * g.nxh;                                                \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 152 * 16) nb = 152 * 16;                                                            \
    sc::specop_kernel<T><<<nb, 256, 0, s>>>(oa, g);                                              \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::rot(const RotArgs<T>& ra, const Geom& g, cudaStream_t s) {          \
    long long n = (long long)g.ny * g.nz * g.nxh;                                                \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 152 * 16) nb = 152 * 16;                                                            \
    sc::rot_update_kernel<T><<<nb, 256, 0, s>>>(ra, g);                                          \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::band_coef(const BandArgs<T>& ba, const Geom& g, cudaStream_t s) {   \
    sc::band_coef_kernel<T><<<1, 256, 0, s>>>(ba, g);                                            \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::ab2v(const Ab2vArgs<T>& aa, const Geom& g, cudaStream_t s) {        \
    long long n = (long long)g.ny * g.nz * g.nxh;                                                \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 152 * 16) nb = 152 * 16;                                                            \
    sc::ab2v_update_kernel<T><<<nb, 256, 0, s>>>(aa, g);                                         \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::moments(const C2<T>* d, const Geom& g, double* partial, int nblocks, \
                                     double* out, cudaStream_t s) {                              \
    const long long rows = (long long)g.ny * g.nz;                                               \
    const int rpb = (int)((rows + nblocks - 1) / nblocks);                                       \
    const int nb = (int)((rows + rpb - 1) / rpb);                                                \
    sc::moments_kernel<T><<<nb, 256, 0, s>>>(d, g, rpb, partial);                                \
    cudaError_t e = cudaGetLastError();                                                          \
    if (e != cudaSuccess) return e;                                                              \
    sc::moments_final_kernel<<<1, 32, 0, s>>>(partial, nb, out);                                 \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::enstrophy(const C2<T>* const w[3], const Geom& g, double* out,       \
                                       cudaStream_t s) {                                         \
    long long n = (long long)g.ny * g.nz * (g.nx / 2);                                           \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 152 * 16) nb = 152 * 16;                                                            \
    sc::enstrophy_kernel<T><<<nb, 256, 0, s>>>(w[0], w[1], w[2], g, out);                        \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::strain(const StrainArgs<T>& sa, const Geom& g, cudaStream_t s) {    \
    long long n = (long long)g.ny * g.nz * g.nxh;                                                \
    int nb = (int)((n + 255) / 256);                                                             \
    if (nb > 152 * 16) nb = 152 * 16;                                                            \
    sc::strain_kernel<T><<<nb, 256, 0, s>>>(sa, g);                                              \
    return cudaGetLastError();                                                                   \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::phys(const PhysArgs<T>& pa, int nblocks, const Geom& g,             \
                                  double* c1_out, double* lm_mm, cudaStream_t s) {               \
    sc::phys_kernel<T><<<nblocks, 256, 0, s>>>(pa, g);                                           \
    cudaError_t e = cudaGetLastError();                                                          \
    if (e != cudaSuccess || pa.op != sc::PH_DYN2) return e;                                      \
    sc::dyn_final_kernel<<<1, 32, 0, s>>>(pa.partial, nblocks, c1_out, lm_mm);                   \
    return cudaGetLastError();                                                                   \
  }

// per-type case bodies (token-pasted above)
#define SC_PLAIN_CASE_float(L) \
  case L: return inv ? sc::launch_plain<float, L, true>(fl, pa, g, nouter, tw, s) \
                     : sc::launch_plain<float, L, false>(fl, pa, g, nouter, tw, s);
#define SC_PLAIN_CASE_double(L) \
  case L: return inv ? sc::launch_plain<double, L, true>(fl, pa, g, nouter, tw, s) \
                     : sc::launch_plain<double, L, false>(fl, pa, g, nouter, tw, s);
#define SC_ZINV_BODY(T, L)                                                      \
  case L:                                                                       \
    switch (mode) {                                                             \
      case sc::ZV_DNS: return sc::launch_zinv<T, L, sc::ZV_DNS>(za, out, g, tw, s);   \
      case sc::ZV_SMAG: return sc::launch_zinv<T, L, sc::ZV_SMAG>(za, out, g, tw, s); \
      case sc::ZV_DYN: return sc::launch_zinv<T, L, sc::ZV_DYN>(za, out, g, tw, s);   \
      case sc::ZV_ADJ: return sc::launch_zinv<T, L, sc::ZV_ADJ>(za, out, g, tw, s);   \
      default: return cudaErrorInvalidValue;                                    \
    }
#define SC_ZINV_CASE_float(L) SC_ZINV_BODY(float, L)
#define SC_ZINV_CASE_double(L) SC_ZINV_BODY(double, L)
#define SC_ZFWD_BODY(T, L)                                                      \
  case L:                                                                       \
    return nin == 9 ? sc::launch_zfwd<T, L, 9>(fin, st, g, tw, s)               \
                    : sc::launch_zfwd<T, L, 3>(fin, st, g, tw, s);
#define SC_ZFWD_CASE_float(L) SC_ZFWD_BODY(float, L)
#define SC_ZFWD_CASE_double(L) SC_ZFWD_BODY(double, L)
#define SC_XPASS_BODY(T, L)                                                           \
  case L:                                                                             \
    switch (mode) {                                                                   \
      case sc::XP_DNS: return sc::launch_xpass<T, L, sc::XP_DNS>(fin, fout, g, twM, twN, xa, s);   \
      case sc::XP_SMAG: return sc::launch_xpass<T, L, sc::XP_SMAG>(fin, fout, g, twM, twN, xa, s); \
      case sc::XP_C2R3: return sc::launch_xpass<T, L, sc::XP_C2R3>(fin, fout, g, twM, twN, xa, s); \
      case sc::XP_R2C3: return sc::launch_xpass<T, L, sc::XP_R2C3>(fin, fout, g, twM, twN, xa, s); \
      case sc::XP_ADJ: return sc::launch_xpass<T, L, sc::XP_ADJ>(fin, fout, g, twM, twN, xa, s);   \
      default: return cudaErrorInvalidValue;                                          \
    }
#define SC_XPASS_CASE_float(L) SC_XPASS_BODY(float, L)
#define SC_XPASS_CASE_double(L) SC_XPASS_BODY(double, L)

#define SC_FUSED_CASE_float(L) \
  case L: return sc::launch_zfwd_zinv<float, L>(lmap, fmap, st, fa, g, tw, err, s);
#define SC_FUSED_CASE_double(L) \
  case L: return sc::launch_zfwd_zinv<double, L>(lmap, fmap, st, fa, g, tw, err, s);
#define SC_ZINV5_CASE_float(L)                                                                     \
  case L:                                                                                          \
    return mode == sc::ZV_SMAG ? sc::launch_zinv5<float, L, sc::ZV_SMAG>(vmap, umap, za, out, g, tw, err, s) \
                               : sc::launch_zinv5<float, L, sc::ZV_DNS>(vmap, umap, za, out, g, tw, err, s);
#define SC_ZINV5_CASE_double(L)                                                                    \
  case L:                                                                                          \
    return mode == sc::ZV_SMAG ? sc::launch_zinv5<double, L, sc::ZV_SMAG>(vmap, umap, za, out, g, tw, err, s) \
                               : sc::launch_zinv5<double, L, sc::ZV_DNS>(vmap, umap, za, out, g, tw, err, s);
#define SC_ZPHI_CASE_float(L) case L: return sc::launch_zinv_phi<float, L>(lmap, omap, za, out, g, tw, err, s);
#define SC_ZPHI_CASE_double(L) case L: return sc::launch_zinv_phi<double, L>(lmap, omap, za, out, g, tw, err, s);
#define SC_ZI_P_CASE_float(L) case L: return sc::ZiCfg<float, L>::P;
#define SC_ZI_P_CASE_double(L) case L: return sc::ZiCfg<double, L>::P;
#define SC_ZI_OK_CASE_float(L) case L: return sc::ZiCfg<float, L>::SUPPORTED;
#define SC_ZI_OK_CASE_double(L) case L: return sc::ZiCfg<double, L>::SUPPORTED;
#define SC_DEFINE_FUSED(T)                                                                       \
  template <> bool sc::Launch<T>::zinv5_supported(int logn) {                                   \
    switch (logn) { SC_LOGN_CASES(SC_ZI_OK_CASE_##T) default: return false; }                    \
  }                                                                                              \
  template <> int sc::Launch<T>::zinv5_tile(int logn) {                                          \
    switch (logn) { SC_LOGN_CASES(SC_ZI_P_CASE_##T) default: return 0; }                         \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zfwd_zinv_tma(int logn, const CUtensorMap& lmap, const CUtensorMap& fmap, \
                                           const StageArgs<T>& st, const FusedArgs<T>& fa,      \
                                           const Geom& g, const C2<T>* tw, int* err,            \
                                           cudaStream_t s) {                                    \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_FUSED_CASE_##T)                                                           \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zinv_phi_tma(int logn, const CUtensorMap& lmap, const CUtensorMap& omap, \
                                          const ZvArgs<T>& za, const FieldList<T>& out, const Geom& g, \
                                          const C2<T>* tw, int* err, cudaStream_t s) {           \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZPHI_CASE_##T)                                                            \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }                                                                                              \
  template <>                                                                                    \
  cudaError_t sc::Launch<T>::zinv5_tma(int logn, const CUtensorMap& vmap, const CUtensorMap& umap, \
                                       const ZvArgs<T>& za, const FieldList<T>& out, const Geom& g, \
                                       const C2<T>* tw, int* err, cudaStream_t s, int mode) {    \
    switch (logn) {                                                                              \
      SC_LOGN_CASES(SC_ZINV5_CASE_##T)                                                           \
      default: return cudaErrorInvalidValue;                                                     \
    }                                                                                            \
  }
