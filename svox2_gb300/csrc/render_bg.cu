// Render kernel instantiations for grids with the MSI background model
// (render_lerp_kernel_cuvol.cu:386-607 and 775-860): the ray march of
// render_core.cuh with the background composited, and differentiated, in the same
// pass as the foreground.  A translation unit of their own, so that they
// compile in parallel with render.cu's.
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

}  // namespace rk
}  // namespace svx
