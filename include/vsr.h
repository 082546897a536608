/*
 * vsr.h -- C ABI of libvsr, the GB300 (sm_103a) focal-stencil library that
 * replaces vibespatial-raster's per-op NVRTC kernels and CuPy launch glue.
 *
 * The reference's operator boundary is its runtime launcher:
 *   get_cuda_runtime().compile_kernels(...) / .launch(kernel=, grid=, block=,
 *   params=(values, types), shared_mem_bytes=)
 * called from src/vibespatial/raster/algebra.py with raw device pointers
 * (CuPy ``.data.ptr``), a nullable uint8 nodata mask, int32 sizes and
 * float64 scalars.  Each entry point below replaces one such launch (plus the
 * float64 up-cast, mask materialisation and down-cast passes around it) and
 * cites the launch it replaces.
 *
 * Conventions
 *   - Every function returns an int status (VSR_OK == 0) and never throws;
 *     vsr_last_error() gives a message for the calling thread.
 *   - The caller owns every buffer.  Pointers are device pointers unless the
 *     parameter name ends in _host.  Pitches are in elements.
 *   - Work is enqueued on ``stream`` (a cudaStream_t, NULL = legacy default
 *     stream) and the call returns without waiting for it, except where a
 *     function says otherwise.
 *   - Distinct streams may be driven from distinct host threads.
 */
#ifndef VSR_H_
#define VSR_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define VSR_API __attribute__((visibility("default")))
#else
#define VSR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define VSR_OK 0
#define VSR_ERR_INVALID_ARG 1  /* bad size, pointer, dtype or parameter     */
#define VSR_ERR_UNSUPPORTED 2  /* valid request this build does not serve  */
#define VSR_ERR_CUDA 3         /* a CUDA runtime/driver call failed         */
#define VSR_ERR_WORKSPACE 4    /* workspace NULL, misaligned or too small   */
#define VSR_ERR_DEVICE 5       /* a kernel reported a device-side error     */

/* ---- element types ----------------------------------------------------- */
#define VSR_U8 1
#define VSR_I16 2
#define VSR_U16 3
#define VSR_I32 4
#define VSR_F32 5
#define VSR_F64 6

/* ---- nodata kinds ------------------------------------------------------ */
#define VSR_NODATA_NONE 0  /* raster has no nodata value                    */
#define VSR_NODATA_VALUE 1 /* pixel == nodata (compared exactly, as float64) */
#define VSR_NODATA_NAN 2   /* pixel is NaN                                  */

/* ---- Horn flags -------------------------------------------------------- */
/* Slope/aspect nodata only at the centre pixel, neighbours' raw values used
 * (the reference GPU kernel, kernels/focal.py:245-262).  Default (flag clear)
 * is the reference CPU rule: any pixel whose 3x3 window touches nodata
 * (algebra.py:2218-2247). */
#define VSR_HORN_CENTER_ONLY 1u
/* Slope/aspect do not mask NaN nodata; NaN propagates through the gradient
 * instead.  This is the reference CPU behaviour (its mask is data == NaN,
 * algebra.py:2188-2189).  Hillshade always masks. */
#define VSR_HORN_SA_NAN_UNMASKED 2u

/* ---- precision for focal convolution -----------------------------------
 * VSR_PREC_SPLIT runs tcgen05 tensor-core GEMMs on split operands with FP32
 * accumulation (hi*hi + hi*lo + lo*hi).  The high parts are BF16; the low
 * part of the data is F16 (11 more bits than BF16, so the dropped lo*lo term
 * is ~2^-20 of a product instead of ~2^-18): the convolution pairs it with
 * an F16 copy of the whole weight, the Gaussian line passes split both sides
 * into F16 pairs.  The two operands of each MMA share one type.
 * VSR_PREC_SPLIT_BF16 is the same code under the name the first builds used. */
#define VSR_PREC_AUTO 0       /* split tensor cores where they pay, else FP32  */
#define VSR_PREC_FP32 1       /* FP32 CUDA-core direct / separable kernels     */
#define VSR_PREC_SPLIT 2      /* tcgen05 split-precision GEMM, FP32 accumulate */
#define VSR_PREC_SPLIT_BF16 VSR_PREC_SPLIT

/* ---- library ------------------------------------------------------------ */
VSR_API int vsr_version(void);                 /* major*10000 + minor*100 + patch      */
VSR_API const char* vsr_last_error(void);      /* message of this thread's last error  */
/* SM count and compute capability of the current device (cudaGetDevice). */
VSR_API int vsr_device_info(int* sm_count, int* cc_major, int* cc_minor);
/* Synchronise ``stream``, then read and clear the device-side error word that
 * kernels set when a bounded wait ran out (0 = none; else an OR of the
 * VSR_DEVERR_* bits below).  Synchronises.  Every spin-wait in a libvsr
 * kernel (on an mbarrier phase that a TMA copy or a tensor-core commit
 * completes) gives up after 2 s, sets its bit, gives the copies it issued a
 * bounded time to land and returns, so the context stays usable. */
#define VSR_DEVERR_TMA_TIMEOUT 1u /* a TMA / cp.async stage never arrived      */
#define VSR_DEVERR_MMA_TIMEOUT 2u /* a tcgen05 commit or TMEM stage never came */
#define VSR_DEVERR_QUEUE 4u       /* a batch work item was out of range        */
#define VSR_DEVERR_PLAN 8u        /* a batch launch disagreed with its plan    */
VSR_API int vsr_poll_device_error(void* stream, uint32_t* code);
/* Exercise the bounded-wait path: one CTA initialises an mbarrier that no
 * copy or thread will ever complete and waits on it with the same bounded
 * wait the kernels use, with a limit of ``limit_ns`` (1e3 .. 2e9 ns) in place
 * of the usual 2 s.  The wait runs out, VSR_DEVERR_TMA_TIMEOUT is raised in
 * the device error word (read it with vsr_poll_device_error) and the kernel
 * writes result[0] = 1 (the wait gave up) and result[1] = the nanoseconds it
 * waited, capped at 2^32 - 1 (``result``: two device uint32 words).  Nothing
 * is in flight when it returns.  No counterpart in the reference. */
VSR_API int vsr_wait_selftest(uint64_t limit_ns, uint32_t* result, void* stream);

/* ---- launch-configuration tuning ----------------------------------------
 * Tunable operations have a small table of launch configurations (tile
 * shape, halo staging depth, threads per CTA, output staging, register
 * budget).  The autotuner
 * (vsr_gb300.autotune) times them on the caller's own data and stores the
 * winner with vsr_tuning_set; the choice is process-wide.  No counterpart in
 * the reference, whose launches use one fixed 16 x 16 block
 * (algebra.py:2323-2338). */
#define VSR_OP_HORN 1
#define VSR_OP_BATCH 2
#define VSR_OP_COUNT 4
VSR_API int vsr_tuning_count(int op);              /* configurations of ``op``; 0 if none */
VSR_API int vsr_tuning_set(int op, int config);
VSR_API int vsr_tuning_get(int op);

/* ---- Horn 3x3: slope / aspect / hillshade in one pass -------------------
 * Replaces the launches of ``slope_aspect`` (algebra.py:2372-2377, kernel
 * kernels/focal.py:173-283) and ``hillshade`` (algebra.py:2748-2754, kernel
 * kernels/focal.py:303-467), plus the float64 up-cast (algebra.py:2283,
 * 2670-2671), the uint8 mask pass (algebra.py:2296-2302, 2687-2696) and the
 * down-cast (algebra.py:2426-2427).  Edge-replicated borders.
 *
 * dem          : height x width raster of ``dtype`` with row pitch ``pitch``
 * cell_x/_y    : |affine a| and |affine e| (1.0 where zero), float64
 * nodata/kind  : nodata value and VSR_NODATA_* kind
 * flags        : VSR_HORN_* bits
 * slope/aspect : outputs in degrees of ``out_dtype`` (VSR_F32 or VSR_F64),
 *                row pitch ``out_pitch``; either may be NULL to skip it.
 *                Nodata pixels receive ``nodata``.
 * hillshade    : uint8 output (row pitch ``hs_pitch``) or NULL; nodata -> 0.
 * z_factor, zenith_rad, azimuth_rad : hillshade parameters; the reference
 *                converts altitude/azimuth degrees to these radians on the
 *                host (algebra.py:2683-2684).
 */
VSR_API int vsr_horn_fused(const void* dem, int dtype, int64_t height, int64_t width, int64_t pitch,
                   double cell_x, double cell_y, double nodata, int nodata_kind, uint32_t flags,
                   void* slope, void* aspect, int out_dtype, int64_t out_pitch,
                   uint8_t* hillshade, int64_t hs_pitch, double z_factor, double zenith_rad,
                   double azimuth_rad, void* stream);

/* Band-first stacks in ONE launch: ``bands`` DEMs ``band_stride`` elements
 * apart; slope/aspect bands ``out_band_stride`` and hillshade bands
 * ``hs_band_stride`` elements apart; otherwise as vsr_horn_fused.  Replaces
 * the per-band loop of dispatch_per_band_gpu (dispatch.py:417-506). */
VSR_API int vsr_horn_fused_bands(const void* dem, int dtype, int bands, int64_t band_stride, int64_t height,
                                 int64_t width, int64_t pitch, double cell_x, double cell_y, double nodata,
                                 int nodata_kind, uint32_t flags, void* slope, void* aspect, int out_dtype,
                                 int64_t out_band_stride, int64_t out_pitch, uint8_t* hillshade,
                                 int64_t hs_band_stride, int64_t hs_pitch, double z_factor, double zenith_rad,
                                 double azimuth_rad, void* stream);

/* ---- terrain derivatives: TRI, TPI, profile curvature -------------------
 * Replaces the ``terrain_derivatives`` launches (algebra.py:2854-2991, kernel
 * kernels/focal.py:487-647), one per derivative, with one pass for any subset,
 * and their float64 up-cast and uint8 mask passes.  Semantics of
 * algebra.py:3352-3445: edge-replicated 3x3 window z0..z8;
 *   TRI = mean |z_i - z4|, TPI = z4 - mean z_i (the 8 neighbours),
 *   curvature = -2 ((z3+z5)/2 - z4)/cx^2 + ((z1+z7)/2 - z4)/cy^2) * 100;
 * border pixels and pixels whose window touches nodata get ``nodata_out``
 * (the reference writes the raster's nodata, else -9999).  Outputs of
 * ``out_dtype`` (the reference returns float64), row pitch ``out_pitch``; any
 * of tri / tpi / curvature may be NULL.  8/16-bit and float32 DEMs are
 * evaluated in double-float FP32 (error-free differences, compensated sums:
 * ~44 significant bits), int32 and float64 DEMs in FP64.
 */
VSR_API int vsr_terrain_derivatives(const void* dem, int dtype, int64_t height, int64_t width, int64_t pitch,
                                    double cell_x, double cell_y, double nodata, int nodata_kind,
                                    double nodata_out, void* tri, void* tpi, void* curvature, int out_dtype,
                                    int64_t out_pitch, void* stream);

/* Band-first stacks in one launch (see vsr_horn_fused_bands). */
VSR_API int vsr_terrain_derivatives_bands(const void* dem, int dtype, int bands, int64_t band_stride, int64_t height,
                                          int64_t width, int64_t pitch, double cell_x, double cell_y, double nodata,
                                          int nodata_kind, double nodata_out, void* tri, void* tpi, void* curvature,
                                          int out_dtype, int64_t out_band_stride, int64_t out_pitch, void* stream);

/* ---- nodata-aware normalised focal convolution --------------------------
 * Replaces the ``convolve_normalized`` launch (algebra.py:2077-2083, kernel
 * kernels/focal.py:36-146) with its up-cast, mask and weight-copy passes
 * (algebra.py:1990-2013).  out[y,x] = sum w*v*valid / sum w*valid over the
 * in-bounds taps of the kh x kw window centred at (kh/2, kw/2), correlation
 * orientation; nodata centre or weight sum <= 0 -> ``nodata`` (pass 0.0 when
 * the raster has none).  A NaN anywhere in the window gives NaN, as in the
 * reference (NaN * 0 = NaN there).
 *
 * weights_host : kh*kw float64 row-major weights in HOST memory
 * precision    : VSR_PREC_*
 * workspace    : device scratch of vsr_convolve_workspace_size() bytes,
 *                256-byte aligned.  The host weights are copied into it with
 *                cudaMemcpyAsync on ``stream`` (so the call returns after the
 *                host copy has been staged) and turned into the kernel's
 *                operand images there by a small float64 prep kernel.
 */
VSR_API size_t vsr_convolve_workspace_size(int kh, int kw, int precision);
VSR_API int vsr_convolve(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch,
                 const double* weights_host, int kh, int kw, double nodata, int nodata_kind,
                 void* dst, int out_dtype, int64_t out_pitch, int precision, void* workspace,
                 size_t workspace_bytes, void* stream);

/* Band-first stacks in one launch (see vsr_horn_fused_bands); the workspace
 * is the same as for one band. */
VSR_API int vsr_convolve_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                               int64_t width, int64_t pitch, const double* weights_host, int kh, int kw,
                               double nodata, int nodata_kind, void* dst, int out_dtype, int64_t out_band_stride,
                               int64_t out_pitch, int precision, void* workspace, size_t workspace_bytes,
                               void* stream);

/* ---- normalised focal convolution that allocates nothing -----------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory and cannot pass a workspace: a serving process whose device memory
 * budget was fixed when it started, or a host that reaches this library
 * through a plugin boundary (ctypes / cgo / JNI) with no access to the
 * process's device allocator.  Same arguments and results as vsr_convolve
 * without the workspace: the scratch is a static device array inside libvsr
 * (358,912 bytes, enough for every kernel up to 80 x 80 at any precision;
 * every GPU that loads the library holds it until the process exits).
 * Larger kernels are rejected with VSR_ERR_UNSUPPORTED.  The first call on
 * each device resolves the array's device address (with that device
 * current); make that first call before any stream capture.  All calls share
 * the one array and it keeps the last call's contents (each call rewrites
 * every scratch byte it reads); calls whose kernels overlap on the GPU (e.g.
 * on two streams at once) race on it.  No cudaMalloc, cudaFree or allocating
 * library routine is called.  ``weights_host`` is staged into the scratch
 * with cudaMemcpyAsync on ``stream``, as in vsr_convolve. */
VSR_API int vsr_convolve_noalloc(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch,
                         const double* weights_host, int kh, int kw, double nodata, int nodata_kind,
                         void* dst, int out_dtype, int64_t out_pitch, int precision, void* stream);

/* ---- Gaussian filter -----------------------------------------------------
 * Replaces raster_gaussian_filter (algebra.py:2120-2154): weights built in
 * float64 on the device (g_i = exp(-0.5 (i - k/2)^2 / sigma^2)); the filter is
 * evaluated separably (row pass held in shared memory, then the column pass),
 * which equals the reference's dense k x k normalised correlation with
 * weights outer(g, g) / sum exactly in real arithmetic, nodata and borders
 * included.  kernel_size <= 0 selects the default 2*ceil(3 sigma)+1; even
 * sizes are bumped to odd.  Same output rule as vsr_convolve.
 *
 * precision: VSR_PREC_FP32 runs the separable FP32 CUDA-core kernels.
 * VSR_PREC_SPLIT runs the two line passes on the tcgen05 tensor cores
 * (8/16-bit integer rasters, kernel_size <= 79): each a GEMM against the
 * Toeplitz band of the split weights (hi*hi + hi*lo + lo*hi, FP32
 * accumulation), the row pass's sums kept as two float32 planes in the
 * workspace.  Its hi/lo pairs are F16 (22 significant bits; a BF16 pair's
 * 16 bits cannot carry the row pass's float32 sums to 2e-6).  VSR_PREC_AUTO takes the tensor cores for such rasters from
 * kernel_size 35 when ``workspace_bytes`` covers
 * vsr_gaussian_workspace_bytes, else the FP32 kernels.
 *
 * vsr_gaussian_workspace_size: the FP32 kernels' workspace (a few KB).
 * vsr_gaussian_workspace_bytes: the workspace for a height x width raster of
 * ``dtype`` at ``precision`` (the tensor-core passes need about 8 bytes per
 * pixel for the row pass's sums).
 * vsr_gaussian_bands_workspace_bytes: the same for a stack of ``bands``
 * rasters run as ONE launch per line pass (the row sums of every band held
 * at once).  vsr_gaussian_bands given less runs the stack in groups of as
 * many bands as the workspace holds, one launch pair per group.
 */
VSR_API size_t vsr_gaussian_workspace_size(int kernel_size, int precision);
VSR_API size_t vsr_gaussian_workspace_bytes(int64_t height, int64_t width, int dtype, double sigma,
                                            int kernel_size, int precision);
VSR_API size_t vsr_gaussian_bands_workspace_bytes(int bands, int64_t height, int64_t width, int dtype, double sigma,
                                                  int kernel_size, int precision);
VSR_API int vsr_gaussian(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch,
                 double sigma, int kernel_size, double nodata, int nodata_kind, void* dst,
                 int out_dtype, int64_t out_pitch, int precision, void* workspace,
                 size_t workspace_bytes, void* stream);

/* Band-first stacks in ONE launch: ``bands`` rasters ``band_stride`` elements
 * apart (output bands ``out_band_stride`` apart), otherwise as vsr_gaussian.
 * Replaces the per-band loop of dispatch_per_band_gpu (dispatch.py:417-506). */
VSR_API int vsr_gaussian_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                       int64_t width, int64_t pitch, double sigma, int kernel_size, double nodata,
                       int nodata_kind, void* dst, int out_dtype, int64_t out_band_stride, int64_t out_pitch,
                       int precision, void* workspace, size_t workspace_bytes, void* stream);

/* ---- focal mean ----------------------------------------------------------
 * Replaces the ``focal_stats`` launch with stat_type 2 (algebra.py:3239-3349,
 * kernel kernels/focal.py:672-769) and the CPU ``_focal_mean_cpu``
 * (algebra.py:3083-3101): mean of the in-bounds, non-nodata, non-NaN values
 * of the (2ry+1) x (2rx+1) window; a nodata centre or an empty window gives
 * ``nodata`` (0.0 when none).  Integer inputs are summed exactly.
 */
VSR_API int vsr_focal_mean(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch,
                   int radius_y, int radius_x, double nodata, int nodata_kind, void* dst,
                   int out_dtype, int64_t out_pitch, void* stream);
/* Band-first stacks in one launch (see vsr_gaussian_bands). */
VSR_API int vsr_focal_mean_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                         int64_t width, int64_t pitch, int radius_y, int radius_x, double nodata,
                         int nodata_kind, void* dst, int out_dtype, int64_t out_band_stride, int64_t out_pitch,
                         void* stream);

/* ---- focal statistics ------------------------------------------------------
 * Replaces the ``focal_stats`` launch (algebra.py:3239-3349, kernel
 * kernels/focal.py:666-770) for every statistic, with the reference CPU
 * functions' semantics (algebra.py:3041-3164, pinned by the oracle):
 *   VSR_STAT_MIN / _MAX  nodata taps excluded, and every tap equal to the
 *                        +inf / -inf placeholder with them (valid +-inf data
 *                        too); a NaN tap gives NaN;
 *   VSR_STAT_MEAN        as vsr_focal_mean;
 *   VSR_STAT_STD         population standard deviation of the valid
 *                        (non-nodata, non-NaN) taps, 0.0 for an empty window;
 *                        exact integer sums for 8/16-bit rasters (a VSR_F32
 *                        output is sqrt(n^2 var)/n rounded once to float32),
 *                        two passes in float64 otherwise;
 *   VSR_STAT_RANGE       max - min of the valid taps;
 *   VSR_STAT_VARIETY     number of distinct valid values, 0 for an empty
 *                        window (no cap; the reference GPU kernel stops at 49).
 * Out-of-bounds taps are excluded.  An empty window gives ``nodata`` (0.0
 * when nodata_kind is VSR_NODATA_NONE); a nodata centre gives ``nodata``.
 * Radii up to 31 (variety: 7); larger ones return VSR_ERR_UNSUPPORTED. */
#define VSR_STAT_MIN 0
#define VSR_STAT_MAX 1
#define VSR_STAT_MEAN 2
#define VSR_STAT_STD 3
#define VSR_STAT_RANGE 4
#define VSR_STAT_VARIETY 5
VSR_API int vsr_focal_stat(const void* src, int dtype, int64_t height, int64_t width, int64_t pitch, int stat,
                           int radius_y, int radius_x, double nodata, int nodata_kind, void* dst, int out_dtype,
                           int64_t out_pitch, void* stream);
/* Band-first stacks in one launch (see vsr_gaussian_bands). */
VSR_API int vsr_focal_stat_bands(const void* src, int dtype, int bands, int64_t band_stride, int64_t height,
                                 int64_t width, int64_t pitch, int stat, int radius_y, int radius_x, double nodata,
                                 int nodata_kind, void* dst, int out_dtype, int64_t out_band_stride,
                                 int64_t out_pitch, void* stream);

/* ---- batched tiles: one persistent launch ------------------------------------
 * Many float32 DEM tiles of uneven sizes, each with its own cell size and
 * nodata, processed by ONE work-queue-scheduled persistent launch: slope and
 * aspect (Horn, as vsr_horn_fused) and a gauss_k x gauss_k Gaussian (as
 * vsr_gaussian) per tile.  Replaces the reference's per-raster / per-band
 * launch loops (dispatch.py:417-506, one launch per band and operation).
 *
 * vsr_batch_plan uploads the tile descriptors into ``plan`` (device memory of
 * vsr_batch_plan_size(n) bytes, 256-byte aligned), builds the Gaussian taps in
 * float64 on the device and synchronises ``stream``.  vsr_batch_run resets the
 * work counter and launches; it makes no host synchronisation and no
 * allocation, so it can be captured in a CUDA graph and replayed.  The plan
 * keeps the tile pointers: replays read and write the same buffers.  The
 * block shape is the tuning table's (VSR_OP_BATCH) when the plan is built;
 * vsr_batch_run launches the plan's own shape whatever the table holds later
 * (re-plan to adopt a new choice), and rejects a ``gauss_k`` other than the
 * plan's, or a plan that vsr_batch_plan did not build in this process. */
typedef struct vsr_batch_tile {
  const float* src;           /* height x width float32, row pitch ``pitch`` */
  int64_t height, width, pitch;
  float* slope;               /* NULL, or with ``aspect``: degrees          */
  float* aspect;
  float* smooth;              /* NULL or the Gaussian output                 */
  int64_t out_pitch;          /* row pitch of the outputs                    */
  double cell_x, cell_y;      /* |affine a|, |affine e| (1.0 where zero)     */
  double nodata;
  int32_t nodata_kind;        /* VSR_NODATA_*                                */
  uint32_t flags;             /* VSR_HORN_* bits                             */
} vsr_batch_tile;

VSR_API size_t vsr_batch_plan_size(int n_tiles);
VSR_API int vsr_batch_plan(const vsr_batch_tile* tiles_host, int n_tiles, double sigma, int gauss_k, void* plan,
                   size_t plan_bytes, int64_t* total_items, void* stream);
VSR_API int vsr_batch_run(void* plan, int gauss_k, void* stream);

/* ---- GeoTIFF decode: chunk assembly on the device -------------------------
 * The device half of reading a GeoTIFF (reference read_raster, io.py:223, and
 * its GPU path nvimgcodec_read, nvimgcodec_io.py:221): the host parses the
 * directory and inflates each chunk (strip or tile) into ``staged`` (device
 * memory, one chunk after another); this call swaps big-endian samples,
 * undoes the predictor (1 none, 2 horizontal differencing in the sample's
 * wrapping integer width, 3 the floating-point byte-plane predictor; 3
 * rewrites ``staged`` in place) and writes every chunk's in-image pixels to
 * the band-first output ``dst`` (bands ``band_stride`` elements apart, rows
 * ``pitch`` elements apart, ``bytes_per_sample`` bytes per element).
 * ``chunks`` (device memory) describes each chunk: its byte offset in
 * ``staged``, the pixel rectangle it covers (its stored width and height;
 * edge tiles may reach past the image) and, for planar-separate files, its
 * band.  Pixel-interleaved samples (``planar`` = 0, up to 4) go to bands
 * 0 .. samples_per_pixel-1. */
typedef struct vsr_tiff_chunk {
  int64_t offset;         /* byte offset of the chunk in ``staged``            */
  int32_t x0, y0;         /* image column and row of its first pixel            */
  int32_t width, height;  /* stored size (tile size, or image width x strip rows) */
  int32_t band;           /* planar-separate files: the chunk's band            */
  int32_t pad_;
} vsr_tiff_chunk;
VSR_API int vsr_tiff_assemble(uint8_t* staged, const vsr_tiff_chunk* chunks, int n_chunks, int max_chunk_rows,
                              int bytes_per_sample, int samples_per_pixel, int planar, int predictor, int big_endian,
                              int64_t height, int64_t width, void* dst, int64_t band_stride, int64_t pitch,
                              void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VSR_H_ */
