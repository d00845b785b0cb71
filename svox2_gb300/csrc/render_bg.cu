// Render kernel instantiations for grids with the MSI background model
// (render_lerp_kernel_cuvol.cu:386-607 and 775-860): the ray march of
// render_core.cuh with the background composited, and differentiated, in the same
// pass as the foreground; the forward kernel of the two-kernel fused step, which also
// runs the background's adjoint; and the SH9 batch kernels whose grids may carry one.
// A translation unit of their own, so that they compile in parallel with
// render.cu's.
#include "render_core.cuh"

namespace svx {
namespace rk {

int dispatch_bg(int mode, bool image, int bd, int dt, const GridP& g, const OptP& opt, const IoP& io,
                long long n, cudaStream_t st) {
  if (mode == kFwd)
    return image ? dispatch_bd<kFwd, true, false, true>(bd, dt, g, opt, io, n, st)
                 : dispatch_bd<kFwd, false, false, true>(bd, dt, g, opt, io, n, st);
  SVX_REQUIRE(!image, SVX_ERR_INVALID, "image renders are forward only");
  if (mode == kFused) return dispatch_bd<kFused, false, false, true>(bd, dt, g, opt, io, n, st);
  return dispatch_bd<kBwd, false, false, true>(bd, dt, g, opt, io, n, st);
}

int launch_bg_split_fwd(int dt, const GridP& g, const OptP& opt, const IoP& io, long long n, cudaStream_t st) {
  switch (dt) {
    case SVX_F32: return launch_t<9, float, kFusedFwd, false, false, true>(g, opt, io, n, st);
    case SVX_BF16: return launch_t<9, __nv_bfloat16, kFusedFwd, false, false, true>(g, opt, io, n, st);
    case SVX_F16: return launch_t<9, __half, kFusedFwd, false, false, true>(g, opt, io, n, st);
  }
  set_error("sh_dtype %d unknown", dt);
  return SVX_ERR_INVALID;
}

int dispatch_bg_batch(int mode, int dt, const GridP& g, const OptP& opt, const IoP& io, long long n,
                      cudaStream_t st) {
  SVX_REQUIRE(mode == kFwd || mode == kFused, SVX_ERR_INVALID, "batch mode %d: render or fused", mode);
  const bool fwd = mode == kFwd;
  switch (dt) {
    case SVX_F32:
      return fwd ? launch_t<9, float, kFwd, false, true, true>(g, opt, io, n, st)
                 : launch_t<9, float, kFused, false, true, true>(g, opt, io, n, st);
    case SVX_BF16:
      return fwd ? launch_t<9, __nv_bfloat16, kFwd, false, true, true>(g, opt, io, n, st)
                 : launch_t<9, __nv_bfloat16, kFused, false, true, true>(g, opt, io, n, st);
    case SVX_F16:
      return fwd ? launch_t<9, __half, kFwd, false, true, true>(g, opt, io, n, st)
                 : launch_t<9, __half, kFused, false, true, true>(g, opt, io, n, st);
  }
  set_error("sh_dtype %d unknown", dt);
  return SVX_ERR_INVALID;
}

}  // namespace rk
}  // namespace svx
