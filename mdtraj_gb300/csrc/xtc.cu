// XTC trajectories decoded on the GPU.
//
// An XTC file is a sequence of XDR (big-endian) frames: magic 1995, atom
// count, step, time, the 3x3 box, the atom count again, then either the raw
// float coordinates (at most 9 atoms) or the compressed form: precision,
// integer bounds minint[3] / maxint[3], the small-integer index, a byte count
// and that many bytes (padded to 4) of a bit stream (formats/xtc/src/
// xdrfile_xtc.c:38-87, xdrfile.c:779-998).  The bit stream encodes, atom by
// atom, the integer coordinates (x * precision, rounded) relative to minint,
// either as three separately sized fields or as one mixed-radix number of
// `sizeofints(sizeint)` bits; a flag bit then announces a new run length (a
// 0 bit repeats the previous one) of following atoms stored as small
// differences (mixed-radix with radix magicints[smallidx]) from the previous
// one, with the first two atoms of a run swapped, and a change of the
// small-integer scale.
//
// gbrmsd_xtc_index scans the frame headers on the host (it only reads
// headers and jumps over the compressed bytes); xtc_decode_kernel decodes one
// frame per thread straight into a padded device coordinate buffer (atom-major,
// the layout of the RMSD kernels).  Every loop is bounded by the frame's byte
// count and atom count; a malformed frame gets a non-zero status and the
// thread stops.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "capi_internal.h"
#include "common.cuh"

namespace gb {
namespace {

constexpr int32_t XTC_MAGIC = 1995;
constexpr int XTC_FIRSTIDX = 9;
constexpr int XTC_NMAGIC = 73;

// The format's table of radices for small integers: values of ~2^(i/3),
// fixed by the file format (xdrfile.c:760-769); entry i is the radix whose
// three-integer mixed-radix number needs i bits.
__constant__ int c_magic[XTC_NMAGIC] = {
    0,        0,        0,       0,       0,       0,       0,       0,       0,       8,        10,
    12,       16,       20,      25,      32,      40,      50,      64,      80,      101,      128,
    161,      203,      256,     322,     406,     512,     645,     812,     1024,    1290,     1625,
    2048,     2580,     3250,    4096,    5060,    6501,    8192,    10321,   13003,   16384,    20642,
    26007,    32768,    41285,   52015,   65536,   82570,   104031,  131072,  165140,  208063,   262144,
    330280,   416127,   524287,  660561,  832255,  1048576, 1321122, 1664510, 2097152, 2642245,  3329021,
    4194304,  5284491,  6658042, 8388607, 10568983, 13316085, 16777216};

enum XtcStatus : int32_t {
  XTC_OK = 0,
  XTC_BAD_MAGIC = 1,
  XTC_BAD_ATOMS = 2,
  XTC_OVERRUN = 3,
  XTC_BAD_INDEX = 4,
};

__host__ __device__ inline uint32_t be32(const uint8_t* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}
__host__ __device__ inline int32_t be_i32(const uint8_t* p) { return (int32_t)be32(p); }
__host__ __device__ inline float be_f32(const uint8_t* p) {
  const uint32_t u = be32(p);
  float f;
  memcpy(&f, &u, 4);
  return f;
}

// MSB-first bit reader over the frame's compressed bytes.
struct BitReader {
  const uint8_t* p;
  uint32_t n;         // bytes available
  uint32_t pos;       // next byte
  uint32_t lastbits;  // unread bits held in lastbyte
  uint32_t lastbyte;
  bool over;
};

__device__ __forceinline__ uint32_t next_byte(BitReader& b) {
  if (b.pos >= b.n) {
    b.over = true;
    return 0;
  }
  return b.p[b.pos++];
}

__device__ __forceinline__ int read_bits(BitReader& b, int nbits) {
  const uint32_t mask = nbits >= 32 ? 0xffffffffu : ((1u << nbits) - 1u);
  uint32_t num = 0;
  while (nbits >= 8) {
    b.lastbyte = (b.lastbyte << 8) | next_byte(b);
    num |= (b.lastbyte >> b.lastbits) << (nbits - 8);
    nbits -= 8;
  }
  if (nbits > 0) {
    if ((int)b.lastbits < nbits) {
      b.lastbits += 8;
      b.lastbyte = (b.lastbyte << 8) | next_byte(b);
    }
    b.lastbits -= nbits;
    num |= (b.lastbyte >> b.lastbits) & ((1u << nbits) - 1u);
  }
  return (int)(num & mask);
}

// Three integers packed as one mixed-radix number of nbits bits (radices
// sizes[0..2], least significant first): read the number as little-endian
// bytes, then peel off the radices from the most significant position down.
__device__ __forceinline__ void read_ints(BitReader& b, int nbits, const uint32_t (&sizes)[3], int (&out)[3]) {
  uint32_t bytes[32];
  bytes[1] = bytes[2] = bytes[3] = 0;
  int nb = 0;
  while (nbits > 8 && nb < 31) {
    bytes[nb++] = (uint32_t)read_bits(b, 8);
    nbits -= 8;
  }
  if (nbits > 0) bytes[nb++] = (uint32_t)read_bits(b, nbits);
  for (int i = 2; i > 0; --i) {
    uint32_t num = 0;
    for (int j = nb - 1; j >= 0; --j) {
      num = (num << 8) | bytes[j];
      const uint32_t q = num / sizes[i];
      bytes[j] = q;
      num -= q * sizes[i];
    }
    out[i] = (int)num;
  }
  out[0] = (int)(bytes[0] | (bytes[1] << 8) | (bytes[2] << 16) | (bytes[3] << 24));
}

// Bits needed for one unsigned value in [0, size) (xdrfile.c:490-501 semantics).
__host__ __device__ inline int bits_of_int(uint32_t size) {
  uint32_t num = 1;
  int bits = 0;
  while (size >= num && bits < 32) {
    ++bits;
    num <<= 1;
  }
  return bits;
}

// Bits of the mixed-radix number of three values with radices sizes[0..2]:
// multiply the radices out in base 256 and count the bits of the product.
__host__ __device__ inline int bits_of_ints(const uint32_t (&sizes)[3]) {
  uint32_t bytes[32];
  int nb = 1;
  bytes[0] = 1;
  for (int i = 0; i < 3; ++i) {
    uint32_t carry = 0;
    int k = 0;
    for (; k < nb; ++k) {
      carry = bytes[k] * sizes[i] + carry;
      bytes[k] = carry & 0xff;
      carry >>= 8;
    }
    while (carry != 0 && k < 32) {
      bytes[k++] = carry & 0xff;
      carry >>= 8;
    }
    nb = k;
  }
  int bits = 0;
  uint32_t num = 1;
  --nb;
  while (bytes[nb] >= num && bits < 32) {
    ++bits;
    num *= 2;
  }
  return bits + nb * 8;
}

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

__device__ __forceinline__ void store3(float* out, int32_t k, float x, float y, float z) {
  out[3 * k] = x;
  out[3 * k + 1] = y;
  out[3 * k + 2] = z;
}

__global__ void __launch_bounds__(128) xtc_decode_kernel(const XtcArgs a) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.n_frames) return;
  const int64_t off = a.offsets[f];
  const uint8_t* p = a.data + off;
  const int64_t avail = a.nbytes - off;
  float* out = a.xyz + f * a.frame_stride;
  int32_t st = XTC_OK;
  const int32_t A = a.n_atoms;
  do {
    if (avail < 56 + 4) { st = XTC_OVERRUN; break; }
    if (be_i32(p) != XTC_MAGIC) { st = XTC_BAD_MAGIC; break; }
    if (be_i32(p + 4) != A || be_i32(p + 52) != A) { st = XTC_BAD_ATOMS; break; }
    if (a.step) a.step[f] = be_i32(p + 8);
    if (a.time) a.time[f] = be_f32(p + 12);
    if (a.box)
      for (int i = 0; i < 9; ++i) a.box[9 * f + i] = be_f32(p + 16 + 4 * i);
    const uint8_t* q = p + 56;
    if (A <= 9) {
      if (avail < 56 + 12 * (int64_t)A) { st = XTC_OVERRUN; break; }
      for (int32_t k = 0; k < A; ++k)
        store3(out, k, be_f32(q + 12 * k), be_f32(q + 12 * k + 4), be_f32(q + 12 * k + 8));
      break;
    }
    if (avail < 56 + 36) { st = XTC_OVERRUN; break; }
    const float precision = be_f32(q);
    int minint[3], maxint[3];
    for (int i = 0; i < 3; ++i) {
      minint[i] = be_i32(q + 4 + 4 * i);
      maxint[i] = be_i32(q + 16 + 4 * i);
    }
    int smallidx = be_i32(q + 28);
    const uint32_t nb = be32(q + 32);
    if (smallidx < XTC_FIRSTIDX || smallidx >= XTC_NMAGIC || (int64_t)nb > avail - 56 - 36) {
      st = smallidx < XTC_FIRSTIDX || smallidx >= XTC_NMAGIC ? XTC_BAD_INDEX : XTC_OVERRUN;
      break;
    }
    BitReader br{q + 36, nb, 0, 0, 0, false};
    uint32_t sizeint[3], bitsizeint[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i) sizeint[i] = (uint32_t)(maxint[i] - minint[i] + 1);
    if (sizeint[0] == 0 || sizeint[1] == 0 || sizeint[2] == 0) { st = XTC_BAD_INDEX; break; }
    int bitsize = 0;
    if ((sizeint[0] | sizeint[1] | sizeint[2]) > 0xffffffu) {
      for (int i = 0; i < 3; ++i) bitsizeint[i] = bits_of_int(sizeint[i]);
    } else {
      bitsize = bits_of_ints(sizeint);
    }
    int smaller = c_magic[max(XTC_FIRSTIDX, smallidx - 1)] / 2;
    int smallnum = c_magic[smallidx] / 2;
    uint32_t sizesmall[3] = {(uint32_t)c_magic[smallidx], (uint32_t)c_magic[smallidx], (uint32_t)c_magic[smallidx]};
    const float inv = (float)(1.0 / (double)precision);
    int32_t k = 0;  // atoms written
    int run = 0;    // a 0 flag bit repeats the previous run length
    while (k < A) {
      int c[3];
      if (bitsize == 0) {
        for (int i = 0; i < 3; ++i) c[i] = read_bits(br, (int)bitsizeint[i]);
      } else {
        read_ints(br, bitsize, sizeint, c);
      }
      for (int i = 0; i < 3; ++i) c[i] += minint[i];
      int prev[3] = {c[0], c[1], c[2]};
      int is_smaller = 0;
      if (read_bits(br, 1) == 1) {
        run = read_bits(br, 5);
        is_smaller = run % 3;
        run -= is_smaller;
        --is_smaller;
      }
      if (br.over || k + 1 + run / 3 > A) { st = XTC_OVERRUN; break; }
      if (run > 0) {
        for (int r = 0; r < run; r += 3) {
          int s[3];
          read_ints(br, smallidx, sizesmall, s);
          for (int i = 0; i < 3; ++i) s[i] += prev[i] - smallnum;
          if (r == 0) {
            // the first two atoms of a run are stored swapped: the first
            // small atom comes out first, the full-size atom second, and
            // later differences are taken from the first small atom
            store3(out, k++, (float)s[0] * inv, (float)s[1] * inv, (float)s[2] * inv);
            store3(out, k++, (float)prev[0] * inv, (float)prev[1] * inv, (float)prev[2] * inv);
            for (int i = 0; i < 3; ++i) prev[i] = s[i];
          } else {
            for (int i = 0; i < 3; ++i) prev[i] = s[i];
            store3(out, k++, (float)s[0] * inv, (float)s[1] * inv, (float)s[2] * inv);
          }
        }
      } else {
        store3(out, k++, (float)c[0] * inv, (float)c[1] * inv, (float)c[2] * inv);
      }
      smallidx += is_smaller;
      if (smallidx < XTC_FIRSTIDX || smallidx >= XTC_NMAGIC) { st = XTC_BAD_INDEX; break; }
      if (is_smaller < 0) {
        smallnum = smaller;
        smaller = smallidx > XTC_FIRSTIDX ? c_magic[smallidx - 1] / 2 : 0;
      } else if (is_smaller > 0) {
        smaller = smallnum;
        smallnum = c_magic[smallidx] / 2;
      }
      sizesmall[0] = sizesmall[1] = sizesmall[2] = (uint32_t)c_magic[smallidx];
      if (br.over) { st = XTC_OVERRUN; break; }
    }
  } while (false);
  if (a.status) a.status[f] = st;
}

// Frame size in bytes at p (0 if the header is malformed or truncated).
int64_t xtc_frame_bytes(const uint8_t* p, int64_t avail, int32_t* natoms) {
  if (avail < 56) return 0;
  if (be_i32(p) != XTC_MAGIC) return 0;
  const int32_t A = be_i32(p + 4);
  if (A < 0 || be_i32(p + 52) != A) return 0;
  *natoms = A;
  if (A <= 9) return 56 + 12 * (int64_t)A <= avail ? 56 + 12 * (int64_t)A : 0;
  if (avail < 56 + 36) return 0;
  const int64_t nb = be32(p + 56 + 32);
  const int64_t sz = 56 + 36 + ((nb + 3) & ~int64_t(3));
  return sz <= avail ? sz : 0;
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
    const int64_t sz = xtc_frame_bytes(data + pos, nbytes - pos, &A);
    if (sz == 0) break;  // truncated tail (or not an XTC frame): stop here
    if (A0 < 0) A0 = A;
    if (A != A0) return set_error(GBRMSD_E_INVALID, "xtc_index: frame %lld has %d atoms, frame 0 has %d", (long long)n, A, A0);
    if (offsets && n < capacity) offsets[n] = pos;
    ++n;
    pos += sz;
  }
  if (n == 0 && nbytes > 0) {
    int32_t A = 0;
    if (nbytes >= 4 && be_i32(data) != XTC_MAGIC) return set_error(GBRMSD_E_INVALID, "xtc_index: not an XTC file (magic)");
    (void)A;
  }
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
