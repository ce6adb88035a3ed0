/*
 * ORACLE — test infrastructure only (never part of the product path).
 *
 * Reads an XTC file with the reference's own C reader (read_xtc,
 * formats/xtc/src/xdrfile_xtc.c, over xdrfile.c's decompression), compiled
 * from the reference's sources by oracle/Makefile into oracle/_ref/: the CPU
 * baseline of the XTC decoding workload and a second check of the GPU decoder.
 */
#include <string.h>

#include "xdrfile.h"
#include "xdrfile_xtc.h"

/* Reads up to max_frames frames of n_atoms atoms; returns the number read
 * (-1 if the file cannot be opened). */
int ref_xtc_read(const char* path, int n_atoms, long max_frames, float* xyz, int* step, float* time, float* box) {
  XDRFILE* xd = xdrfile_open(path, "r");
  if (!xd) return -1;
  long n = 0;
  while (n < max_frames) {
    int st = 0;
    float t = 0.0f, prec = 0.0f;
    matrix b;
    if (read_xtc(xd, n_atoms, &st, &t, b, (rvec*)(xyz + 3L * n_atoms * n), &prec) != exdrOK) break;
    if (step) step[n] = st;
    if (time) time[n] = t;
    if (box) memcpy(box + 9 * n, b, sizeof(matrix));
    ++n;
  }
  xdrfile_close(xd);
  return (int)n;
}
