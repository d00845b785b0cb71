/*
 * svox2_gb300 — C ABI of the GB300-native (sm_103a) Plenoxels sparse-voxel renderer.
 *
 * Every entry point takes plain pointers and sizes, never a framework tensor.
 * All data pointers are DEVICE pointers on the current CUDA device unless a
 * field says otherwise; `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Every call is asynchronous on `stream`, returns an
 * svx_status (0 = success) and leaves a one-line message for
 * svx_last_error() on failure (thread-local).  Kernel launches are checked
 * with cudaGetLastError; faults inside a kernel surface at the caller's next
 * synchronisation.
 *
 * Each function replaces one operator of the reference's `svox2.csrc`
 * extension (pybind11 table in svox2/csrc/svox2.cpp:74-112); the comment above
 * each declaration names the reference declaration and implementation it
 * stands in for.  Argument meaning follows the reference; where the reference
 * passed a torch::Tensor, the ABI passes its device pointer plus the sizes the
 * reference read from the tensor.
 */
#ifndef SVOX2_GB300_H_
#define SVOX2_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SVX_ABI_VERSION 3

/* Status codes.  The reference raised RuntimeError through TORCH_CHECK
 * (svox2/csrc/include/data_spec.hpp:32-51); the ABI returns these instead and
 * the Python layer raises RuntimeError with svx_last_error(). */
typedef enum {
  SVX_OK = 0,
  SVX_ERR_INVALID = 1,      /* bad argument: null pointer, size, dtype, range */
  SVX_ERR_UNSUPPORTED = 2,  /* feature this library does not implement (MLP basis, 3D texture…) */
  SVX_ERR_CUDA = 3,         /* a CUDA runtime call or kernel launch failed */
  SVX_ERR_TOO_LARGE = 4     /* size beyond a documented limit */
} svx_status;

/* Storage type of a float table (SH coefficients, TV/optimiser data). */
typedef enum { SVX_F32 = 0, SVX_BF16 = 1, SVX_F16 = 2 } svx_dtype;

/* Basis types, svox2/defs.py:1-4.  Only SVX_BASIS_SH is built. */
#define SVX_BASIS_SH 1
#define SVX_BASIS_3D_TEXTURE 4
#define SVX_BASIS_MLP 255

/* Grid description — SparseGridSpec, svox2/csrc/include/data_spec.hpp:18-52,
 * packed form svox2/csrc/include/data_spec_packed.cuh:11-62.
 *   links      int32 [size0, size1, size2], C-contiguous; >= 0 is a row index
 *              into the data tables, -1 is empty, < -1 is an empty-space skip
 *              level written by accel_dist_prop.
 *   density    float32 [n_voxels, 1].
 *   sh         [n_voxels, sh_data_dim] of sh_dtype, channel-major per voxel:
 *              coefficient k of colour channel c is sh[v, c*basis_dim + k];
 *              4-byte aligned (rows are copied in aligned 4-byte words).
 *   offset/scaling  world -> grid transform, grid = world*scaling + offset
 *              (the reference's _offset/_scaling CPU tensors, svox2/svox2.py:2135-2161).
 *   background_nlayers  0, or the layer count (>= 2) of the MSI background model
 *              (svox2/svox2.py:497-521), whose tables are:
 *   background_links  int32 [2 * background_reso, background_reso], C-contiguous;
 *              >= 0 is a row of background_data, < 0 is empty.
 *   background_data   float32 [background_capacity, background_nlayers, 4], 16-byte
 *              aligned: per layer three colour coefficients (scaled by the SH DC
 *              constant) and sigma.  A link >= background_capacity reads as empty.
 * The MSI background is rendered by the ray entry points (cuvol.cu:386-607) and by
 * svx_render_batch when its with_background flag is set; svx_ray_order and the
 * depth renders ignore it, as the reference's depth renders do. */
typedef struct {
  const float* density_data;
  const void* sh_data;
  const int32_t* links;
  int64_t n_voxels;
  int32_t size[3];
  int32_t basis_dim;
  int32_t sh_data_dim;
  int32_t basis_type;
  int32_t sh_dtype;
  int32_t background_nlayers;
  float offset[3];
  float scaling[3];
  const int32_t* background_links;
  const float* background_data;
  int64_t background_capacity;
  int32_t background_reso;
} svx_grid_t;

/* RaysSpec, data_spec.hpp:104-113: origins and unit directions, float32 [n_rays, 3]. */
typedef struct {
  const float* origins;
  const float* dirs;
  int64_t n_rays;
} svx_rays_t;

/* CameraSpec, data_spec.hpp:83-102.  c2w is a DEVICE float32 row-major matrix
 * with 4 columns and c2w_rows (3 or 4) rows, OpenCV convention. */
typedef struct {
  const float* c2w;
  int32_t c2w_rows;
  float fx, fy, cx, cy;
  int32_t width, height;
  float ndc_coeffx, ndc_coeffy;
} svx_camera_t;

/* RenderOptions, data_spec.hpp:115-135. */
typedef struct {
  float background_brightness;
  float step_size;
  float sigma_thresh;
  float stop_thresh;
  float near_clip;
  int32_t use_spheric_clip;
  int32_t last_sample_opaque;
} svx_render_opts_t;

/* GridOutputGrads, data_spec.hpp:54-81.  Gradients are float32 and are
 * ACCUMULATED into (not overwritten).  mask_out (bool/uint8 [n_voxels]) may be
 * NULL; when given, every voxel that received a gradient is set to 1.
 * grad_background_out (float32 [capacity, nlayers, 4]) and mask_background_out
 * (bool/uint8 [capacity, nlayers]) are the MSI background's, used when the grid
 * has one; either may be NULL. */
typedef struct {
  float* grad_density_out;
  float* grad_sh_out;
  uint8_t* mask_out;
  float* grad_background_out;
  uint8_t* mask_background_out;
} svx_grid_grads_t;

/* Optional instrumentation for the render entry points (may be NULL):
 *   eval_samples  device uint64 accumulator: += number of evaluated samples
 *                 (sigma > sigma_thresh, before early stop) over the launch.
 *   ray_trace     device uint64 [n_rays]: per-ray hash of the sequence of
 *                 (cell, links, evaluated) decisions; lets tests compare the
 *                 sample indexing bit for bit with a CPU restatement.
 *   march_start, march_stop
 *                 cudaEvent_t handles of the caller (or NULL), recorded on the
 *                 call's stream just before and just after the ray-march kernel,
 *                 so that its duration can be told apart from the ray sort and
 *                 the gradient flush around it.
 *   background_samples  device uint64 accumulator: += number of MSI background
 *                 samples (sigma > 0, before early stop) over the launch. */
typedef struct {
  uint64_t* eval_samples;
  uint64_t* ray_trace;
  void* march_start;
  void* march_stop;
  uint64_t* background_samples;
} svx_render_stats_t;

/* ---- rendering: svox2/csrc/render_lerp_kernel_cuvol.cu ---------------- */

/* volume_render_cuvol (svox2/csrc/svox2.cpp:18, render_lerp_kernel_cuvol.cu:918-958).
 * rgb_out float32 [n_rays, 3]. */
int svx_volume_render_cuvol(const svx_grid_t* grid, const svx_rays_t* rays,
                            const svx_render_opts_t* opt, float* rgb_out,
                            const svx_render_stats_t* stats, void* stream);

/* volume_render_cuvol_image (svox2/csrc/svox2.cpp:19-20, render_lerp_kernel_cuvol.cu:960-1008).
 * rgb_out float32 [height, width, 3]. */
int svx_volume_render_cuvol_image(const svx_grid_t* grid, const svx_camera_t* cam,
                                  const svx_render_opts_t* opt, float* rgb_out,
                                  const svx_render_stats_t* stats, void* stream);

/* volume_render_cuvol_backward (svox2/csrc/svox2.cpp:21-22, render_lerp_kernel_cuvol.cu:1010-1068).
 * grad_out = dL/d(rgb) float32 [n_rays, 3].  color_cache is the forward
 * output; it is accepted for interface parity and may be NULL, because this
 * adjoint rebuilds what it needs from the grid.  Gradients accumulate into
 * grads; the reference does not set the mask on this path, neither does this. */
int svx_volume_render_cuvol_backward(const svx_grid_t* grid, const svx_rays_t* rays,
                                     const svx_render_opts_t* opt, const float* grad_out,
                                     const float* color_cache, const svx_grid_grads_t* grads,
                                     const svx_render_stats_t* stats, void* stream);

/* volume_render_cuvol_fused (svox2/csrc/svox2.cpp:23-24, render_lerp_kernel_cuvol.cu:1070-1152).
 * Renders rgb_out [n_rays,3] and accumulates the gradient of
 * mean((rgb_out - rgb_gt)^2) (+ beta_loss, sparsity_loss terms) into grads,
 * setting grads->mask_out for every touched voxel.
 * Scratch comes from the device's default stream-ordered pool.  For an SH9 grid the step runs
 * as two kernels with a record per ray between them (24 * cap + 32 bytes, cap = the grid's
 * longest ray in samples rounded up to 32: 21.5 KB a ray at 256^3, step 0.5); the records of one
 * call take at most SVX_FUSED_SPLIT_BYTES bytes (environment variable, read at each call;
 * default 24 GiB), larger calls run in chunks of rays, 0 selects the one-kernel form, and so does
 * a pool that cannot supply the records. */
int svx_volume_render_cuvol_fused(const svx_grid_t* grid, const svx_rays_t* rays,
                                  const svx_render_opts_t* opt, const float* rgb_gt,
                                  float beta_loss, float sparsity_loss, float* rgb_out,
                                  const svx_grid_grads_t* grads,
                                  const svx_render_stats_t* stats, void* stream);

/* volume_render_expected_term (svox2/csrc/svox2.cpp:25, render_lerp_kernel_cuvol.cu:122-176,
 * 862-880, 1154-1172): out float32 [n_rays], the expected termination distance of each
 * ray in world units, sum over evaluated samples of weight * (t / step_size) * world_step
 * (0 for a ray that misses the grid). */
int svx_volume_render_expected_term(const svx_grid_t* grid, const svx_rays_t* rays,
                                    const svx_render_opts_t* opt, float* out, void* stream);

/* volume_render_sigma_thresh (svox2/csrc/svox2.cpp:26, render_lerp_kernel_cuvol.cu:178-225,
 * 882-902, 1174-1195): out float32 [n_rays], the distance of the first sample whose
 * density exceeds sigma_thresh (0 if none). */
int svx_volume_render_sigma_thresh(const svx_grid_t* grid, const svx_rays_t* rays,
                                   const svx_render_opts_t* opt, float sigma_thresh, float* out,
                                   void* stream);

/* svx_volume_render_cuvol_fused_noalloc — no counterpart in the reference.
 * The fused render above for callers that cannot allocate device memory
 * while they run (work inside another framework's callbacks, hosts that plan
 * all device memory up front, processes whose device heap belongs to a
 * foreign allocator).  Same arguments and results as
 * svx_volume_render_cuvol_fused; it calls no cudaMalloc/cudaFree and no
 * allocating routine.  Its scratch (the ray counter) is a 256-byte static
 * device array held by every GPU that loads the library until exit; a call
 * needs 8 bytes of it whatever the number of rays or the grid's size, which
 * the library checks against the array when it is compiled.  The first call
 * on a device looks the array's address up (again after a device reset) and
 * should come before any stream capture on that device.  All calls share the
 * array: calls that overlap on the GPU race on the counter and must be
 * serialised by the caller. */
int svx_volume_render_cuvol_fused_noalloc(const svx_grid_t* grid, const svx_rays_t* rays,
                                          const svx_render_opts_t* opt, const float* rgb_gt,
                                          float beta_loss, float sparsity_loss, float* rgb_out,
                                          const svx_grid_grads_t* grads,
                                          const svx_render_stats_t* stats, void* stream);

/* ---- serving: batched launches over several resident grids -------------
 * No counterpart in the reference (it renders one grid per call).  A serving
 * loop puts the rays of several requests, on several resident grids, into one
 * persistent launch.  All grids of a batch share basis_dim and sh_dtype. */

/* One grid of a batch, read by the kernel from DEVICE memory.  For the fused
 * mode: where this grid's gradients go (accum: optional padded rows
 * [n_voxels][accum_stride], accum_stride a multiple of 4 >= sh_data_dim + 1,
 * zeroed by the caller, added into the gradients by the caller), and the MSE
 * scale norm = 2 / (3 * rays of this grid's request) with the beta / sparsity
 * loss weights (beta already divided by that ray count). */
typedef struct {
  svx_grid_t grid;
  svx_grid_grads_t grads;
  float* accum;
  int32_t accum_stride;
  float norm;
  float beta;
  float sparsity;
} svx_batch_grid_t;

/* Render (mode 0) or fused-MSE render (mode 1) of a batch of rays.
 *   grids       device array of svx_batch_grid_t; the host does not read it,
 *               so the caller vouches for it (pointers, sizes, basis_dim; an
 *               MSI background's table and gradient 16-byte aligned)
 *   with_background  0: every grid is rendered without its MSI background
 *               (a faster kernel); 1: grids whose background_nlayers > 0 are
 *               rendered, and in mode 1 differentiated, with it
 *   ray_grid    device int32 [max_rays], the grid of each ray
 *   n_rays_dev  device int64: rays processed by this launch (<= max_rays); it
 *               is read on the device, so that a captured CUDA graph of this
 *               call can be replayed for a new batch after the buffers change
 *   order       NULL (rays in index order) or device int32 [max_rays]: the i-th
 *               ray processed is order[i]; the first n_rays entries must be a
 *               permutation of 0..n_rays-1 (see svx_ray_order).  Outputs stay
 *               at each ray's own index.
 *   work        device uint64 scratch of the caller (cleared by the call)
 *   colour_cache  NULL, or device memory of colour_cache_bytes (16-byte
 *               aligned) for the fused mode.  At least
 *               svx_batch_record_bytes(max_rays, n) bytes (n >= 64), without
 *               the MSI background: the step runs as two kernels with a record
 *               of n samples per ray there, and rays with more evaluated
 *               samples are redone by the one-kernel step.  Otherwise, at least
 *               svx_batch_colour_cache_bytes(n) bytes (n >= 32): the one-kernel
 *               step keeps each ray's per-sample colours there for its reverse
 *               pass.  Without it the cache is 48 samples in shared memory, and
 *               longer rays gather their colours again.
 * Allocates nothing.  max_rays sizes the persistent grid. */
int svx_render_batch(int32_t mode, const svx_batch_grid_t* grids, int32_t basis_dim, int32_t sh_dtype,
                     int32_t with_background, const float* origins, const float* dirs, const int32_t* ray_grid,
                     const int32_t* order, const int64_t* n_rays_dev, int64_t max_rays,
                     const svx_render_opts_t* opt, const float* rgb_gt, float* rgb_out, uint64_t* work,
                     float* colour_cache, int64_t colour_cache_bytes, void* stream);

/* Bytes of a svx_render_batch colour cache that holds samples_per_ray
 * evaluated samples for every warp the batch launch keeps resident on the
 * current device (16 bytes a sample). */
int64_t svx_batch_colour_cache_bytes(int32_t samples_per_ray);

/* Bytes of a svx_render_batch colour cache that holds, for each of max_rays
 * rays, a record of samples_per_ray evaluated samples (rounded up to 32; 24
 * bytes a sample and a 32-byte header), after a 16-byte counter and an int32
 * list of max_rays entries.  No counterpart in the reference. */
int64_t svx_batch_record_bytes(int64_t max_rays, int32_t samples_per_ray);

/* Coherence order of a ray table against one grid: order_out[i] = index_base +
 * the index of the i-th ray sorted by (octahedral direction bucket, Morton code
 * of the chord midpoint inside the grid); rays that miss the grid go last.  This
 * is the order the fused render uses internally for large batches; a caller that
 * packs several requests into one svx_render_batch uses it per request.  Uses
 * stream-ordered scratch (about 16 bytes per ray plus the sort's own). */
int svx_ray_order(const svx_grid_t* grid, const svx_rays_t* rays, const svx_render_opts_t* opt,
                  int32_t index_base, int32_t* order_out, void* stream);

/* grad_sh[v, c] += accum[v, c] and grad_density[v] += accum[v, sh_data_dim] for
 * every row v < n_voxels of a padded accumulation table [n_voxels, stride]
 * (the accum of svx_batch_grid_t); rows that are all zero are skipped, so the
 * untouched gradients keep their exact values.  Either output may be NULL. */
int svx_add_accum(const float* accum, int32_t stride, int32_t sh_data_dim, int64_t n_voxels, float* grad_sh,
                  float* grad_density, void* stream);

/* The rays of a pinhole camera (what volume_render_cuvol_image marches,
 * cam2world_ray in svox2/csrc/include/render_util.cuh:526-544), written as
 * origins / dirs float32 [height * width, 3] in row-major pixel order. */
int svx_camera_rays(const svx_camera_t* cam, float* origins, float* dirs, void* stream);

/* ---- point sampling: svox2/csrc/svox2_kernel.cu ------------------------ */

/* sample_grid (svox2/csrc/svox2.cpp:11-12, svox2_kernel.cu:181-217).
 * points float32 [n_points, 3] in world coordinates (grid->offset/scaling
 * apply).  out_density float32 [n_points, 1]; out_sh float32
 * [n_points, sh_data_dim], written only when want_colors != 0. */
int svx_sample_grid(const svx_grid_t* grid, const float* points, int64_t n_points,
                    int32_t want_colors, float* out_density, float* out_sh, void* stream);

/* sample_grid_backward (svox2/csrc/svox2.cpp:13-14, svox2_kernel.cu:219-267).
 * Accumulates into grad_density_out [n_voxels,1] and (want_colors)
 * grad_sh_out [n_voxels, sh_data_dim]. */
int svx_sample_grid_backward(const svx_grid_t* grid, const float* points, int64_t n_points,
                             const float* grad_out_density, const float* grad_out_sh,
                             float* grad_density_out, float* grad_sh_out,
                             int32_t want_colors, void* stream);

/* ---- total variation: svox2/csrc/loss_kernel.cu ------------------------ */

/* A float table [n_rows, n_cols] of data_dtype (density or SH). */
typedef struct {
  const void* data;
  int32_t dtype;
  int64_t n_rows;
  int32_t n_cols;
} svx_table_t;

/* tv (svox2/csrc/svox2.cpp:60, loss_kernel.cu:42-109, host 483-515).  Writes
 * to the device float *out the TV value of channels [start_dim, end_dim): the mean
 * over the (size0-1)(size1-1)(size2-1) cells of sqrt(1e-5 + |d * size/256|^2),
 * summed over channels.  use_logalpha must be 0 (the reference rejects it too). */
int svx_tv(const int32_t* links, const int32_t size[3], const svx_table_t* data, int32_t start_dim,
           int32_t end_dim, int32_t use_logalpha, float logalpha_delta, int32_t ignore_edge,
           float ndc_coeffx, float ndc_coeffy, float* out, void* stream);

/* tv_grad (svox2/csrc/svox2.cpp:62-63, loss_kernel.cu:111-176, host 522-556).
 * Dense TV gradient over all (size0-1)(size1-1)(size2-1) cells, channels
 * [start_dim, end_dim), scaled by scale / n_cells, accumulated into grad
 * (float32 [n_rows, n_cols]).  use_logalpha/logalpha_delta are accepted and
 * unused, as in the reference. */
int svx_tv_grad(const int32_t* links, const int32_t size[3], const svx_table_t* data,
                int32_t start_dim, int32_t end_dim, float scale, int32_t use_logalpha,
                float logalpha_delta, int32_t ignore_edge, float ndc_coeffx,
                float ndc_coeffy, float* grad, void* stream);

/* tv_grad_sparse (svox2/csrc/svox2.cpp:64-65, loss_kernel.cu:178-246, host 558-604).
 * TV gradient on the n_cells linear cell indices rand_cells (int32), scaled
 * by scale / n_cells; sets mask_out[v] = 1 for every voxel written (mask_out
 * may be NULL). */
int svx_tv_grad_sparse(const int32_t* links, const int32_t size[3], const svx_table_t* data,
                       const int32_t* rand_cells, int64_t n_cells, uint8_t* mask_out,
                       int32_t start_dim, int32_t end_dim, float scale, int32_t use_logalpha,
                       float logalpha_delta, int32_t ignore_edge, int32_t ignore_last_z,
                       float ndc_coeffx, float ndc_coeffy, float* grad, void* stream);

/* msi_tv_grad_sparse (svox2/csrc/svox2.cpp:66, loss_kernel.cu:248-333, host 606-641).
 * TV gradient of the MSI background on the n_cells cell indices rand_cells
 * (int32, index = (x * reso + y) * nlayers + z over the [2 reso, reso, nlayers]
 * cells): differences to the next cell in x and y wrap around, in z they stop
 * at the last layer.  Channels 0..n_channels-2 are scaled by scale / n_cells,
 * the last (sigma) by scale_last / n_cells.  links int32 [2 reso, reso] (a link
 * >= capacity reads as empty); msi and grad float32 [capacity, nlayers,
 * n_channels]; mask_out (uint8 [capacity, nlayers]) may be NULL.  Cell indices
 * outside the MSI are skipped. */
int svx_msi_tv_grad_sparse(const int32_t* links, int32_t reso, const float* msi, int64_t capacity,
                           int32_t nlayers, int32_t n_channels, const int32_t* rand_cells, int64_t n_cells,
                           uint8_t* mask_out, float scale, float scale_last, float* grad, void* stream);

/* ---- optimisers: svox2/csrc/optim_kernel.cu ---------------------------- */

/* How the optimiser selects rows: the reference dispatched on the indexer
 * tensor (optim_kernel.cu:168-216): 0-dim -> all rows, empty -> nothing,
 * bool [n_rows] -> mask, int64 [n] -> row list. */
typedef enum {
  SVX_INDEX_ALL = 0,
  SVX_INDEX_NONE = 1,
  SVX_INDEX_MASK = 2,   /* indexer: const uint8_t* [n_rows] */
  SVX_INDEX_LIST = 3    /* indexer: const int64_t* [n_index] */
} svx_indexer_kind;

/* rmsprop_step (svox2/csrc/svox2.cpp:70-71, optim_kernel.cu:154-218).
 * data [n_rows, n_cols] of data_dtype (updated in place; f32, bf16 or f16),
 * rms and grad float32 [n_rows, n_cols]; grad is zeroed on the visited rows.
 * lr_last < 0 means lr_last = lr.  The last column uses lr_last. */
int svx_rmsprop_step(void* data, int32_t data_dtype, float* rms, float* grad,
                     int64_t n_rows, int32_t n_cols, int32_t indexer_kind,
                     const void* indexer, int64_t n_index, float beta, float lr,
                     float epsilon, float minval, float lr_last, void* stream);

/* sgd_step (svox2/csrc/svox2.cpp:72, optim_kernel.cu:220-267). */
int svx_sgd_step(void* data, int32_t data_dtype, float* grad, int64_t n_rows,
                 int32_t n_cols, int32_t indexer_kind, const void* indexer,
                 int64_t n_index, float lr, float lr_last, void* stream);

/* ---- empty-space skipping: svox2/csrc/misc_kernel.cu ------------------- */

/* accel_dist_prop (svox2/csrc/svox2.cpp:54, misc_kernel.cu:108-181 and 356-416;
 * SparseGrid.accelerate, svox2/svox2.py:1487-1494).  Rewrites, in place, every
 * negative entry of the int32 links table [size0, size1, size2] as -(1 + e), e
 * being the number of consecutive empty levels (no voxel with a link >= 0)
 * above the voxel in a pyramid that halves each side, rounding up, while all
 * sides are > 1.  Entries >= 0 are unchanged.  Uses stream-ordered scratch of
 * about 1/7 byte per voxel. */
int svx_accel_dist_prop(int32_t* links, const int32_t size[3], void* stream);

/* dilate (svox2/csrc/svox2.cpp:53, misc_kernel.cu:20-48 and 335-350): out[v] =
 * OR of the bool/uint8 grid [size0, size1, size2] over the 3x3x3 block around v,
 * clamped at the faces.  out must not alias grid. */
int svx_dilate(const uint8_t* grid, uint8_t* out, const int32_t size[3], void* stream);

/* grid_weight_render (svox2/csrc/svox2.cpp:55-57, misc_kernel.cu:183-334 and 418-448):
 * marches every pixel ray of cam through the dense float32 density grid data
 * [size0, size1, size2] (world -> grid: grid = world * scaling + offset, host
 * floats) and raises grid_weight (float32, same shape, >= 0 on entry) at the 8
 * corners of each sample with sigma > 1e-8 to that sample's rendering weight. */
int svx_grid_weight_render(const float* data, const int32_t size[3], const svx_camera_t* cam, float step_size,
                           float stop_thresh, int32_t last_sample_opaque, const float offset[3],
                           const float scaling[3], float* grid_weight, void* stream);

/* ---- library ------------------------------------------------------------ */

/* Message of the last failed call on this thread ("" if none). */
const char* svx_last_error(void);

/* SVX_ABI_VERSION of the loaded library. */
int svx_abi_version(void);

/* Largest number of evaluated samples per ray whose colours the adjoint keeps
 * in shared memory when it has no global colour cache (the allocation-free
 * render and the batch launch); samples past it are re-gathered in the
 * reverse pass.  The fused and backward renders keep a global cache as long
 * as the grid's longest ray (up to 4096 samples). */
int svx_color_cache_capacity(void);

#ifdef __cplusplus
}
#endif

#endif /* SVOX2_GB300_H_ */
