// XTC trajectories decoded on the GPU.
//
// gbrmsd_xtc_index scans the frame headers on the host (it only reads
// headers and jumps over the compressed bytes); xtc_decode_kernel decodes one
// frame per thread straight into a padded device coordinate buffer (atom-major,
// the layout of the RMSD kernels) with the decoder of xtc_dec.cuh (the format
// and the bit reader are described there).  A malformed frame gets a
// non-zero status and its thread stops.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "capi_internal.h"
#include "common.cuh"
#include "xtc_dec.cuh"

namespace gb {
namespace {

struct XtcArgs {
  const uint8_t* data;
  int64_t nbytes;
  const int64_t* offsets;
  int64_t n_frames;
  int32_t n_atoms;
  float* xyz;
  int64_t frame_stride;
  int32_t* step;
  float* time;
  float* box;
  int32_t* status;
};

__global__ void __launch_bounds__(128) xtc_decode_kernel(const XtcArgs a) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.n_frames) return;
  const int32_t st = xtc::decode_frame(a.data, a.nbytes, a.offsets[f], a.n_atoms, a.xyz + f * a.frame_stride,
                                       a.step ? a.step + f : nullptr, a.time ? a.time + f : nullptr,
                                       a.box ? a.box + 9 * f : nullptr);
  if (a.status) a.status[f] = st;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gbrmsd_xtc_index(const uint8_t* data, int64_t nbytes, int64_t* offsets, int64_t capacity, int64_t* n_frames,
                     int32_t* n_atoms, int64_t* consumed) {
  clear_error();
  if ((!data && nbytes > 0) || nbytes < 0 || !n_frames || !n_atoms)
    return set_error(GBRMSD_E_INVALID, "xtc_index: null arguments");
  int64_t pos = 0, n = 0;
  int32_t A0 = -1;
  while (pos < nbytes) {
    int32_t A = 0;
    const int64_t sz = xtc::frame_bytes(data + pos, nbytes - pos, &A);
    if (sz == 0) break;  // truncated tail (or not an XTC frame): stop here
    if (A0 < 0) A0 = A;
    if (A != A0) return set_error(GBRMSD_E_INVALID, "xtc_index: frame %lld has %d atoms, frame 0 has %d", (long long)n, A, A0);
    if (offsets && n < capacity) offsets[n] = pos;
    ++n;
    pos += sz;
  }
  if (n == 0 && nbytes >= 4 && xtc::be_i32(data) != xtc::MAGIC)
    return set_error(GBRMSD_E_INVALID, "xtc_index: not an XTC file (magic)");
  *n_frames = n;
  *n_atoms = A0 < 0 ? 0 : A0;
  if (consumed) *consumed = pos;
  return GBRMSD_OK;
}

int gbrmsd_xtc_decode(const uint8_t* data, int64_t nbytes, const int64_t* offsets, int64_t n_frames, int32_t n_atoms,
                      float* xyz, int64_t frame_stride, int32_t* step, float* time, float* box, int32_t* status,
                      void* stream) {
  clear_error();
  if (n_frames < 0 || n_atoms < 0 || frame_stride < 3LL * n_atoms)
    return set_error(GBRMSD_E_INVALID, "xtc_decode: bad sizes");
  if (n_frames == 0) return GBRMSD_OK;
  if (!data || !offsets || (!xyz && n_atoms > 0)) return set_error(GBRMSD_E_INVALID, "xtc_decode: null pointer");
  XtcArgs a{data, nbytes, offsets, n_frames, n_atoms, xyz, frame_stride, step, time, box, status};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_begin(st);
  xtc_decode_kernel<<<(unsigned)((n_frames + 127) / 128), 128, 0, st>>>(a);
  GB_CUDA_TRY(cudaGetLastError(), "launch xtc_decode_kernel");
  prof_end(st);
  return GBRMSD_OK;
}

}  // extern "C"
