// GeoTIFF decode, device side: the step between the decompressed chunk bytes
// and the raster the stencils read (reference: read_raster, io.py:223, whose
// GPU path is nvimgcodec_read, nvimgcodec_io.py:221).
//
// The host parses the TIFF directory and inflates the chunks (strips or
// tiles) into one staging buffer; vsr_tiff_assemble then, on the GPU, for
// every chunk row (one thread per row, or per row and sample):
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

// One thread per (chunk, chunk row); grid-stride over all of them.
__global__ void tiff_assemble_kernel(const TiffArgs a) {
  const int64_t total = static_cast<int64_t>(a.n_chunks) * a.max_rows;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int ci = static_cast<int>(t / a.max_rows), r = static_cast<int>(t - static_cast<int64_t>(ci) * a.max_rows);
    const vsr_tiff_chunk c = a.chunks[ci];
    if (r >= c.height) continue;
    const int64_t y = static_cast<int64_t>(c.y0) + r;
    const int ns = a.planar ? 1 : a.spp;  // samples interleaved in this chunk
    const int64_t row_vals = static_cast<int64_t>(c.width) * ns;
    uint8_t* row = a.staged + c.offset + static_cast<int64_t>(r) * row_vals * a.esz;
    const int64_t ncols = c.x0 + static_cast<int64_t>(c.width) <= a.W ? c.width : a.W - c.x0;
    if (a.predictor == 3) {
      // byte planes: undo the byte-wise differencing over the whole row, then
      // value i's bytes are plane b at i (b = 0 most significant)
      const int64_t nb = row_vals * a.esz;
      for (int64_t i = 1; i < nb; ++i) row[i] = static_cast<uint8_t>(row[i] + row[i - 1]);
      if (y >= a.H) continue;
      for (int64_t x = 0; x < ncols; ++x)
        for (int s = 0; s < ns; ++s) {
          const int64_t i = x * ns + s;
          uint64_t v = 0;
          for (int b = 0; b < a.esz; ++b) v = (v << 8) | row[b * row_vals + i];
          const int band = a.planar ? c.band : s;
          store_elem(a.dst + (band * a.band_stride + y * a.pitch + c.x0 + x) * a.esz, a.esz, v);
        }
      continue;
    }
    if (y >= a.H) continue;
    uint64_t acc[4] = {0, 0, 0, 0};
    const uint64_t mask = a.esz == 8 ? ~0ull : ((1ull << (8 * a.esz)) - 1ull);
    for (int64_t x = 0; x < ncols; ++x)
      for (int s = 0; s < ns; ++s) {
        uint64_t v = load_elem(row + (x * ns + s) * a.esz, a.esz, a.swap);
        if (a.predictor == 2) {  // wrapping sum in the sample's own width
          const int k = s < 4 ? s : 3;
          acc[k] = (acc[k] + v) & mask;
          v = acc[k];
        }
        const int band = a.planar ? c.band : s;
        store_elem(a.dst + (band * a.band_stride + y * a.pitch + c.x0 + x) * a.esz, a.esz, v);
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
  const int64_t total = static_cast<int64_t>(n_chunks) * max_chunk_rows;
  const int threads = 128;
  const int64_t blocks = std::min<int64_t>((total + threads - 1) / threads, static_cast<int64_t>(sm_count()) * 16);
  tiff_assemble_kernel<<<static_cast<unsigned>(blocks > 0 ? blocks : 1), threads, 0, static_cast<cudaStream_t>(stream)>>>(a);
  VSR_CUDA_TRY(cudaGetLastError());
  return VSR_OK;
}
