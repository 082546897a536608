// GeoTIFF decode, device side: the step between the decompressed chunk bytes
// and the raster the stencils read (reference: read_raster, io.py:223, whose
// GPU path is nvimgcodec_read, nvimgcodec_io.py:221).
//
// The host parses the TIFF directory and inflates the chunks (strips or
// tiles) into one staging buffer; vsr_tiff_assemble then, on the GPU, for
// every chunk row (one warp per row, its lanes over the row's values):
//   * swaps the bytes of big-endian files,
//   * undoes the predictor: 2 = horizontal differencing, a running sum per
//     sample in the sample's own wrapping integer type; 3 = the floating-point
//     predictor, byte-wise differencing over the row's byte planes (most
//     significant plane first) then the planes interleaved back into values,
//   * writes the chunk's pixels that lie inside the image into the band-first
//     (B, H, W) output (partial edge tiles clipped; pixel-interleaved samples
//     go to their bands).
#include "vsr_internal.cuh"

namespace vsr {
namespace {

__device__ __forceinline__ uint64_t load_elem(const uint8_t* p, int esz, bool swap) {
  uint64_t v = 0;
  for (int b = 0; b < esz; ++b) v |= static_cast<uint64_t>(p[swap ? esz - 1 - b : b]) << (8 * b);
  return v;
}

__device__ __forceinline__ void store_elem(uint8_t* p, int esz, uint64_t v) {
  for (int b = 0; b < esz; ++b) p[b] = static_cast<uint8_t>(v >> (8 * b));
}

struct TiffArgs {
  uint8_t* staged;  // decompressed chunks (modified in place by predictor 3)
  const vsr_tiff_chunk* chunks;
  int n_chunks;
  int esz, spp, planar, predictor, swap;
  int64_t H, W;
  uint8_t* dst;
  int64_t band_stride, pitch;  // elements
  int max_rows;                // largest chunk height
};

// Inclusive prefix sum of one value per lane over the warp (wrapping in
// the value's width is the caller's mask).
__device__ __forceinline__ uint64_t warp_scan(uint64_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

// One warp per (chunk, chunk row), grid-stride over all of them.  Lanes
// take consecutive values, so loads and stores are coalesced; the running
// sums of the predictors are warp scans carried from one 32-value step to
// the next.
__global__ void tiff_assemble_kernel(const TiffArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  const int64_t total = static_cast<int64_t>(a.n_chunks) * a.max_rows;
  for (int64_t t = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; t < total; t += warps) {
    const int ci = static_cast<int>(t / a.max_rows), r = static_cast<int>(t - static_cast<int64_t>(ci) * a.max_rows);
    const vsr_tiff_chunk c = a.chunks[ci];
    if (r >= c.height) continue;
    const int64_t y = static_cast<int64_t>(c.y0) + r;
    const int ns = a.planar ? 1 : a.spp;  // samples interleaved in this chunk
    const int64_t row_vals = static_cast<int64_t>(c.width) * ns;
    uint8_t* row = a.staged + c.offset + static_cast<int64_t>(r) * row_vals * a.esz;
    const int64_t ncols = c.x0 + static_cast<int64_t>(c.width) <= a.W ? c.width : a.W - c.x0;
    if (a.predictor == 3) {
      // byte planes: undo the byte-wise differencing over the whole row (a
      // wrapping byte scan, 32 lanes x 4 bytes per step), then value i's
      // bytes are plane b at i (b = 0 most significant)
      const int64_t nb = row_vals * a.esz;
      uint32_t carry = 0;
      for (int64_t b0 = 0; b0 < nb; b0 += 128) {
        const int64_t i0 = b0 + 4 * lane;
        uint32_t v0 = 0, v1 = 0, v2 = 0, v3 = 0;
        if (i0 + 0 < nb) v0 = row[i0 + 0];
        if (i0 + 1 < nb) v1 = row[i0 + 1];
        if (i0 + 2 < nb) v2 = row[i0 + 2];
        if (i0 + 3 < nb) v3 = row[i0 + 3];
        v1 += v0;
        v2 += v1;
        v3 += v2;
        const uint32_t incl = static_cast<uint32_t>(warp_scan(v3, lane));
        const uint32_t excl = incl - v3 + carry;
        if (i0 + 0 < nb) row[i0 + 0] = static_cast<uint8_t>(v0 + excl);
        if (i0 + 1 < nb) row[i0 + 1] = static_cast<uint8_t>(v1 + excl);
        if (i0 + 2 < nb) row[i0 + 2] = static_cast<uint8_t>(v2 + excl);
        if (i0 + 3 < nb) row[i0 + 3] = static_cast<uint8_t>(v3 + excl);
        carry += __shfl_sync(0xffffffffu, incl, 31);
      }
      __syncwarp();
      if (y >= a.H) continue;
      for (int64_t i = lane; i < ncols * ns; i += 32) {
        uint64_t v = 0;
        for (int b = 0; b < a.esz; ++b) v = (v << 8) | row[b * row_vals + i];
        const int64_t x = i / ns;
        const int s = static_cast<int>(i - x * ns);
        const int band = a.planar ? c.band : s;
        store_elem(a.dst + (band * a.band_stride + y * a.pitch + c.x0 + x) * a.esz, a.esz, v);
      }
      continue;
    }
    if (y >= a.H) continue;
    const uint64_t mask = a.esz == 8 ? ~0ull : ((1ull << (8 * a.esz)) - 1ull);
    for (int s = 0; s < ns; ++s) {
      const int band = a.planar ? c.band : s;
      uint8_t* orow = a.dst + (band * a.band_stride + y * a.pitch + c.x0) * a.esz;
      uint64_t carry = 0;
      for (int64_t x0 = 0; x0 < ncols; x0 += 32) {
        const int64_t x = x0 + lane;
        uint64_t v = x < ncols ? load_elem(row + (x * ns + s) * a.esz, a.esz, a.swap) : 0;
        if (a.predictor == 2) {  // running sum of the differences, wrapping in the sample's width
          const uint64_t incl = warp_scan(v, lane);
          v = (incl + carry) & mask;
          carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (x < ncols) store_elem(orow + x * a.esz, a.esz, v);
      }
    }
  }
}

}  // namespace
}  // namespace vsr

using namespace vsr;

extern "C" int vsr_tiff_assemble(uint8_t* staged, const vsr_tiff_chunk* chunks, int n_chunks, int max_chunk_rows,
                                 int bytes_per_sample, int samples_per_pixel, int planar, int predictor,
                                 int big_endian, int64_t height, int64_t width, void* dst, int64_t band_stride,
                                 int64_t pitch, void* stream) {
  if (n_chunks < 0 || max_chunk_rows < 0 || height < 0 || width < 0) return fail(VSR_ERR_INVALID_ARG, "negative size");
  if (n_chunks == 0 || height == 0 || width == 0) return VSR_OK;
  if (!staged || !chunks || !dst) return fail(VSR_ERR_INVALID_ARG, "staged/chunks/dst must not be NULL");
  if (bytes_per_sample != 1 && bytes_per_sample != 2 && bytes_per_sample != 4 && bytes_per_sample != 8)
    return fail(VSR_ERR_UNSUPPORTED, "bytes per sample must be 1, 2, 4 or 8");
  if (samples_per_pixel < 1 || samples_per_pixel > 4)
    return fail(VSR_ERR_UNSUPPORTED, "1 to 4 samples per pixel are supported");
  if (predictor != 1 && predictor != 2 && predictor != 3) return fail(VSR_ERR_UNSUPPORTED, "TIFF predictor %d", predictor);
  if (pitch < width || (samples_per_pixel > 1 && band_stride < pitch * height))
    return fail(VSR_ERR_INVALID_ARG, "output pitch / band stride too small");
  TiffArgs a{staged, chunks, n_chunks, bytes_per_sample, samples_per_pixel, planar ? 1 : 0, predictor,
             big_endian ? 1 : 0, height, width, static_cast<uint8_t*>(dst), band_stride, pitch, max_chunk_rows};
  const int64_t total = static_cast<int64_t>(n_chunks) * max_chunk_rows;  // one warp each
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>((total * 32 + threads - 1) / threads, static_cast<int64_t>(sm_count()) * 16);
  tiff_assemble_kernel<<<static_cast<unsigned>(blocks > 0 ? blocks : 1), threads, 0, static_cast<cudaStream_t>(stream)>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}
