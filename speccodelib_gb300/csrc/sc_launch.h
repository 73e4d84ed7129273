// Host-side launch interface of the pass kernels, one specialisation per
// arithmetic type (float: FP32-bulk mode, double: plain FP64 mode).  Each
// launcher dispatches the runtime axis length to a compiled template
// instance; lengths outside 8..1024 return cudaErrorInvalidValue.
#pragma once
#include <cuda.h>

#include "sc_common.cuh"

namespace sc {

// Lane-major twiddle tables of the warp FFT, after the 4096-entry table of
// power-of-two lengths: for M = 32 E (LOGM 5 .. 9) a block of 1024 entries
// at 4096 + 1024 (LOGM - 5) holding W_M^{j lane} at (j - 1) 32 + lane and
// W_M^{j q E} at (E - 1) 32 + (j - 1) Q + q (j = 1 .. E-1, lane < 32,
// q < Q = 32 / E).
struct WarpTw {
  static constexpr int BASE = 4096, BLOCK = 1024, LOGM_MIN = 5, LOGM_MAX = 9;
  static constexpr int TOTAL = BASE + BLOCK * (LOGM_MAX - LOGM_MIN + 1);
  __host__ __device__ static constexpr int offset(int logm) { return BASE + BLOCK * (logm - LOGM_MIN); }
  __host__ __device__ static constexpr bool covers(int logm) { return logm >= LOGM_MIN && logm <= LOGM_MAX; }
  // The whole table (TOTAL entries, host side): entry L + m = e^{-2 pi i m/L}
  // for L = 2 .. 2048 (computed in double precision, then rounded), then the
  // lane-major blocks as copies of those entries.
  template <typename C, typename FC, typename FS> static void fill(C* t, FC cosf_, FS sinf_) {
    for (int i = 0; i < 4; ++i) t[i] = C{};
    for (int L = 2; L <= 2048; L *= 2)
      for (int m = 0; m < L; ++m) {
        const double a = 2.0 * 3.14159265358979323846 * (double)m / (double)L;
        t[L + m].x = (decltype(t[0].x))cosf_(a);
        t[L + m].y = (decltype(t[0].x))(-sinf_(a));
      }
    t[0] = t[1] = C{};
    for (int logm = LOGM_MIN; logm <= LOGM_MAX; ++logm) {
      const int M = 1 << logm, E = M / 32, Q = 32 / E;
      C* b = t + offset(logm);
      for (int j = 1; j < E; ++j) {
        for (int lane = 0; lane < 32; ++lane) b[(j - 1) * 32 + lane] = t[M + (lane * j) % M];
        for (int q = 0; q < Q; ++q) b[(E - 1) * 32 + (j - 1) * Q + q] = t[M + (q * E * j) % M];
      }
    }
  }
};

template <typename T> struct PlainArgs;
template <typename T> struct ZvArgs;
template <typename T> struct StageArgs;
template <typename T> struct XArgs;
template <typename T> struct DiagArgs;
template <typename T> struct SpecOpArgs;
template <typename T> struct RotArgs;
template <typename T> struct Ab2vArgs;
template <typename T> struct StrainArgs;
template <typename T> struct PhysArgs;
template <typename T> struct TmaPass;
template <typename T> struct AdjArgs;
template <typename T> struct AdjOpArgs;
template <typename T> struct FusedArgs;
template <typename T> struct BandArgs;

template <typename T> struct Launch {
  static int tile();                                   // pencil tile width P
  // strided-axis pass: grid = (ceil(nxh/P), nouter)
  static cudaError_t plain(int logn, bool inverse, const FieldList<T>& fl, const PlainArgs<T>& pa,
                           const Geom& g, int nouter, const C2<T>* tw, cudaStream_t s);
  static cudaError_t zinv_vel(int logn, int mode, const ZvArgs<T>& za, const FieldList<T>& out,
                              const Geom& g, const C2<T>* tw, cudaStream_t s);
  static cudaError_t zfwd_stage(int logn, int nin, const FieldList<T>& fin, const StageArgs<T>& st,
                                const Geom& g, const C2<T>* tw, cudaStream_t s);
  static cudaError_t fixup(const StageArgs<T>& st, const Geom& g, cudaStream_t s);
  static cudaError_t xpass(int logm, int mode, const FieldList<T>& fin, const FieldList<T>& fout,
                           const Geom& g, const C2<T>* twM, const C2<T>* twN, const XArgs<T>& xa,
                           cudaStream_t s);
  // spectral-space elementwise operators and reductions (sc_ops.cuh)
  static cudaError_t diag(const DiagArgs<T>& da, const Geom& g, cudaStream_t s);
  static cudaError_t specop(const SpecOpArgs<T>& oa, const Geom& g, cudaStream_t s);
  // helical-wave AB2 update of the rotating solver at every mode
  static cudaError_t rot(const RotArgs<T>& ra, const Geom& g, cudaStream_t s);
  // force_rot's coefficient into *ba.out on the device (one block)
  static cudaError_t band_coef(const BandArgs<T>& ba, const Geom& g, cudaStream_t s);
  // variable-step IF-AB2 update at every mode
  static cudaError_t ab2v(const Ab2vArgs<T>& aa, const Geom& g, cudaStream_t s);
  static cudaError_t strain(const StrainArgs<T>& sa, const Geom& g, cudaStream_t s);
  // post-processing of physical packed rows: sums of d^2, d^3 into out[0..1]
  // (partial holds 2 doubles per block, nblocks at most); enstrophy density
  // 1/2 |w|^2 into a real (nz, ny, nx) array
  static cudaError_t moments(const C2<T>* d, const Geom& g, double* partial, int nblocks, double* out,
                             cudaStream_t s);
  static cudaError_t enstrophy(const C2<T>* const w[3], const Geom& g, double* out, cudaStream_t s);
  // physical-space pointwise op; PH_DYN2 also finishes cs2 into *c1_out
  static cudaError_t phys(const PhysArgs<T>& pa, int nblocks, const Geom& g, double* c1_out,
                          double* lm_mm, cudaStream_t s);
  // TMA-fed strided passes (sc_tma_passes.cuh).  Tile widths and box extent
  // the host needs to encode the tensor maps:
  static int tma_tile(int logn);       // pencil_tma / zfwd_tma tile width
  static int tma_ztile(int logn);      // zinv_tma tile width
  static cudaError_t plain_tma(int logn, bool inverse, const CUtensorMap& map, const TmaPass<T>& tp,
                               const Geom& g, const C2<T>* tw, int nsm, cudaStream_t s);
  static cudaError_t zinv_tma(int logn, const CUtensorMap& vmap, const ZvArgs<T>& za,
                              const FieldList<T>& out, const Geom& g, const C2<T>* tw, int* err,
                              cudaStream_t s);
  // vstore (RK stage 4 only): the new state leaves by bulk tensor stores
  // through vmap (st.vout[0..2], tiles as lmap)
  static cudaError_t zfwd_tma(int logn, const CUtensorMap& lmap, const CUtensorMap& vmap, int vstore,
                              const StageArgs<T>& st, const Geom& g, const C2<T>* tw, int* err, cudaStream_t s);
  // z-forward of nin fields (9: the LES Lamb vector and tau_ij) through a
  // TMA ring, fmap tiled tma_tile wide; cudaErrorNotSupported otherwise
  static cudaError_t zfwd_fields_tma(int logn, int nin, const CUtensorMap& fmap, const StageArgs<T>& st,
                                     const Geom& g, const C2<T>* tw, int* err, cudaStream_t s);
  // z-inverse of the DNS operands with five transforms from TMA-loaded stage
  // input tiles, and the z-forward pass of RK stages 1-3 fused with it
  // (sc_fused.cuh), tile width zinv5_tile.  zinv5_supported: whether the
  // tiles fit shared memory for this length (else cudaErrorNotSupported).
  static bool zinv5_supported(int logn);
  static int zinv5_tile(int logn);     // tile width of zinv5 / zinv_phi / zfwd_zinv
  // umap: a map of out.f[0..2] tiled zinv5_tile wide, used when
  // za.ustore (u leaves by bulk tensor stores)
  // mode ZV_DNS = 0 (u, w) or ZV_SMAG (u, w, S_ij: eight transforms, not 12)
  static cudaError_t zinv5_tma(int logn, const CUtensorMap& vmap, const CUtensorMap& umap, const ZvArgs<T>& za,
                               const FieldList<T>& out, const Geom& g, const C2<T>* tw, int* err,
                               cudaStream_t s, int mode = 0);
  // phi^ of the adjoint right-hand side from TMA-loaded lam tiles (za.lam is
  // unused; the map covers lam), with the forcing-adjoint band sums; with
  // za.ustore, at 256- and 512-point pencils, phi leaves by bulk tensor
  // stores through omap (out's three fields, tiles as lmap), else by element
  // stores to out
  static cudaError_t zinv_phi_tma(int logn, const CUtensorMap& lmap, const CUtensorMap& omap, const ZvArgs<T>& za,
                                  const FieldList<T>& out, const Geom& g, const C2<T>* tw, int* err,
                                  cudaStream_t s);
  // fmap: the whole field slab, tiles as lmap, for the L2 prefetch of the
  // update operands (StageArgs::pf_slot)
  static cudaError_t zfwd_zinv_tma(int logn, const CUtensorMap& lmap, const CUtensorMap& fmap,
                                   const StageArgs<T>& st, const FusedArgs<T>& fa, const Geom& g,
                                   const C2<T>* tw, int* err, cudaStream_t s);
  // discrete adjoint (sc_adjoint.cuh)
  static cudaError_t zfwd_adj(int logn, const FieldList<T>& fin, const AdjArgs<T>& aa, const Geom& g,
                              const C2<T>* tw, cudaStream_t s);
  // the same, the six product tiles by TMA (tma_tile width); fidx maps the
  // kernel's field order (w x phi, phi x u) to the tensor map's fields
  static int adj_tile(int logn);       // zfwd_adj_tma tile width (its pmap's)
  static cudaError_t zfwd_adj_tma(int logn, const CUtensorMap& pmap, const int fidx[6], const AdjArgs<T>& aa,
                                  const Geom& g, const C2<T>* tw, int* err, cudaStream_t s);
  static cudaError_t adj_copyT(const FieldList<T>& lw, const Geom& g, cudaStream_t s);
  static cudaError_t adj_op(const AdjOpArgs<T>& ao, const Geom& g, cudaStream_t s);
  // warp-per-row x-pass (sc_xwarp.cuh): mode XW_DNS (Lamb product), XW_ADJ
  // (its adjoint) or XW_SMAG (Lamb product and Smagorinsky tau_ij);
  // cudaErrorNotSupported for lengths it has no instance for
  static cudaError_t xpass_warp(int logm, int mode, const FieldList<T>& fin, const FieldList<T>& fout,
                                const Geom& g, const C2<T>* twM, const C2<T>* twN, const XArgs<T>& xa,
                                cudaStream_t s);
};

}  // namespace sc
