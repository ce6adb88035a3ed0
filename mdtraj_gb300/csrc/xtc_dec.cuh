// XTC frame decoder shared by the GPU kernel (xtc.cu) and a host build that
// tests it on the CPU against the reference reader's output.
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
#pragma once

#include <stdint.h>
#include <string.h>

namespace gb {
namespace xtc {

constexpr int32_t MAGIC = 1995;
constexpr int FIRSTIDX = 9;
constexpr int NMAGIC = 73;

enum Status : int32_t {
  OK = 0,
  BAD_MAGIC = 1,
  BAD_ATOMS = 2,
  OVERRUN = 3,
  BAD_INDEX = 4,
};

// The format's table of radices for small integers: values of ~2^(i/3),
// fixed by the file format (xdrfile.c:760-769); entry i is the radix whose
// three-integer mixed-radix number needs i bits.  One copy in constant
// memory for the GPU, one for the host build.
#define GB_XTC_MAGIC_TABLE                                                                                   \
  {0,        0,        0,       0,       0,       0,       0,       0,       0,       8,        10,           \
   12,       16,       20,      25,      32,      40,      50,      64,      80,      101,      128,          \
   161,      203,      256,     322,     406,     512,     645,     812,     1024,    1290,     1625,         \
   2048,     2580,     3250,    4096,    5060,    6501,    8192,    10321,   13003,   16384,    20642,        \
   26007,    32768,    41285,   52015,   65536,   82570,   104031,  131072,  165140,  208063,   262144,       \
   330280,   416127,   524287,  660561,  832255,  1048576, 1321122, 1664510, 2097152, 2642245,  3329021,      \
   4194304,  5284491,  6658042, 8388607, 10568983, 13316085, 16777216}
__constant__ int c_magic[NMAGIC] = GB_XTC_MAGIC_TABLE;
static const int h_magic[NMAGIC] = GB_XTC_MAGIC_TABLE;
#undef GB_XTC_MAGIC_TABLE

__host__ __device__ inline int magic(int i) {
#ifdef __CUDA_ARCH__
  return c_magic[i];
#else
  return h_magic[i];
#endif
}

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
  const uint8_t* p;   // first byte of the stream
  uint32_t n;         // bytes available
  uint32_t pos;       // next byte
  uint32_t lastbits;  // unread bits held in lastbyte
  uint32_t lastbyte;
  bool over;
};

__host__ __device__ inline uint32_t next_byte(BitReader& b) {
  if (b.pos >= b.n) {
    b.over = true;
    return 0;
  }
  return b.p[b.pos++];
}

__host__ __device__ inline int read_bits(BitReader& b, int nbits) {
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
// sizes[0..2], least significant first): the number is read as
// little-endian bytes, and out[2] = x mod sizes[2], out[1] = (x / sizes[2])
// mod sizes[1], out[0] = the low 32 bits of the rest.  Numbers of up to 32
// or 64 bits (every small-difference atom and most full-size ones) are
// divided as one integer in registers; longer ones by the byte-wise long
// division of the format's reader.
__host__ __device__ inline void read_ints(BitReader& b, int nbits, const uint32_t (&sizes)[3], int (&out)[3]) {
  if (nbits <= 32) {
    uint32_t x = 0;
    int sh = 0;
    for (; nbits > 8; nbits -= 8, sh += 8) x |= (uint32_t)read_bits(b, 8) << sh;
    if (nbits > 0) x |= (uint32_t)read_bits(b, nbits) << sh;
    out[2] = (int)(x % sizes[2]);
    x /= sizes[2];
    out[1] = (int)(x % sizes[1]);
    out[0] = (int)(x / sizes[1]);
    return;
  }
  if (nbits <= 64) {
    uint64_t x = 0;
    int sh = 0;
    for (; nbits > 8; nbits -= 8, sh += 8) x |= (uint64_t)read_bits(b, 8) << sh;
    if (nbits > 0) x |= (uint64_t)read_bits(b, nbits) << sh;
    out[2] = (int)(x % sizes[2]);
    x /= sizes[2];
    out[1] = (int)(x % sizes[1]);
    out[0] = (int)(uint32_t)(x / sizes[1]);
    return;
  }
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

__host__ __device__ inline void store3(float* out, int32_t k, float x, float y, float z) {
  out[3 * k] = x;
  out[3 * k + 1] = y;
  out[3 * k + 2] = z;
}

// Decodes the frame at data + off (of a buffer of nbytes bytes) with A atoms
// into out[0 .. 3A) (atom-major floats); step / time / box (9 floats) are
// written when non-null.  Returns a Status.  Every loop is bounded by the
// frame's byte count and atom count.
__host__ __device__ inline int32_t decode_frame(const uint8_t* data, int64_t nbytes, int64_t off, int32_t A,
                                                float* out, int32_t* step, float* time, float* box) {
  const uint8_t* p = data + off;
  const int64_t avail = nbytes - off;
  if (avail < 56 + 4) return OVERRUN;
  if (be_i32(p) != MAGIC) return BAD_MAGIC;
  if (be_i32(p + 4) != A || be_i32(p + 52) != A) return BAD_ATOMS;
  if (step) *step = be_i32(p + 8);
  if (time) *time = be_f32(p + 12);
  if (box)
    for (int i = 0; i < 9; ++i) box[i] = be_f32(p + 16 + 4 * i);
  const uint8_t* q = p + 56;
  if (A <= 9) {
    if (avail < 56 + 12 * (int64_t)A) return OVERRUN;
    for (int32_t k = 0; k < A; ++k) store3(out, k, be_f32(q + 12 * k), be_f32(q + 12 * k + 4), be_f32(q + 12 * k + 8));
    return OK;
  }
  if (avail < 56 + 36) return OVERRUN;
  const float precision = be_f32(q);
  int minint[3], maxint[3];
  for (int i = 0; i < 3; ++i) {
    minint[i] = be_i32(q + 4 + 4 * i);
    maxint[i] = be_i32(q + 16 + 4 * i);
  }
  int smallidx = be_i32(q + 28);
  const uint32_t nb = be32(q + 32);
  if (smallidx < FIRSTIDX || smallidx >= NMAGIC) return BAD_INDEX;
  if ((int64_t)nb > avail - 56 - 36) return OVERRUN;
  BitReader br{q + 36, nb, 0, 0, 0, false};
  uint32_t sizeint[3], bitsizeint[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i) sizeint[i] = (uint32_t)(maxint[i] - minint[i] + 1);
  if (sizeint[0] == 0 || sizeint[1] == 0 || sizeint[2] == 0) return BAD_INDEX;
  int bitsize = 0;
  if ((sizeint[0] | sizeint[1] | sizeint[2]) > 0xffffffu) {
    for (int i = 0; i < 3; ++i) bitsizeint[i] = bits_of_int(sizeint[i]);
  } else {
    bitsize = bits_of_ints(sizeint);
  }
  int smaller = magic(smallidx - 1 > FIRSTIDX ? smallidx - 1 : FIRSTIDX) / 2;
  int smallnum = magic(smallidx) / 2;
  uint32_t sizesmall[3] = {(uint32_t)magic(smallidx), (uint32_t)magic(smallidx), (uint32_t)magic(smallidx)};
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
    if (br.over || k + 1 + run / 3 > A) return OVERRUN;
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
    if (smallidx < FIRSTIDX || smallidx >= NMAGIC) return BAD_INDEX;
    if (is_smaller < 0) {
      smallnum = smaller;
      smaller = smallidx > FIRSTIDX ? magic(smallidx - 1) / 2 : 0;
    } else if (is_smaller > 0) {
      smaller = smallnum;
      smallnum = magic(smallidx) / 2;
    }
    sizesmall[0] = sizesmall[1] = sizesmall[2] = (uint32_t)magic(smallidx);
    if (br.over) return OVERRUN;
  }
  return OK;
}

// Frame size in bytes at p (0 if the header is malformed or truncated).
__host__ __device__ inline int64_t frame_bytes(const uint8_t* p, int64_t avail, int32_t* natoms) {
  if (avail < 56) return 0;
  if (be_i32(p) != MAGIC) return 0;
  const int32_t A = be_i32(p + 4);
  if (A < 0 || be_i32(p + 52) != A) return 0;
  *natoms = A;
  if (A <= 9) return 56 + 12 * (int64_t)A <= avail ? 56 + 12 * (int64_t)A : 0;
  if (avail < 56 + 36) return 0;
  const int64_t nb = be32(p + 56 + 32);
  const int64_t sz = 56 + 36 + ((nb + 3) & ~int64_t(3));
  return sz <= avail ? sz : 0;
}

}  // namespace xtc
}  // namespace gb
