// Host build of the GPU's XTC frame decoder (mdtraj_gb300/csrc/xtc_dec.cuh):
// decodes every frame of the XTC file named on the command line and writes,
// per frame, the status (int32), step (int32), time (float32), box (9
// float32) and coordinates (3 x n_atoms float32) to stdout, after a header of
// two int64 (frames, atoms).  The test compares them with the reference
// reader's output.  With a second argument the whole file is first copied to
// that byte offset of a larger buffer (other alignments of the stream).
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "../mdtraj_gb300/csrc/xtc_dec.cuh"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  FILE* fp = fopen(argv[1], "rb");
  if (!fp) return 3;
  std::vector<uint8_t> raw;
  uint8_t buf[65536];
  size_t got;
  while ((got = fread(buf, 1, sizeof buf, fp)) > 0) raw.insert(raw.end(), buf, buf + got);
  fclose(fp);
  const int64_t shift = argc > 2 ? atoll(argv[2]) : 0;
  std::vector<uint8_t> store(raw.size() + shift + 16);
  uint8_t* data = store.data() + shift;
  for (size_t i = 0; i < raw.size(); ++i) data[i] = raw[i];
  const int64_t nbytes = (int64_t)raw.size();
  std::vector<int64_t> offs;
  int32_t A0 = -1;
  for (int64_t pos = 0; pos < nbytes;) {
    int32_t A = 0;
    const int64_t sz = gb::xtc::frame_bytes(data + pos, nbytes - pos, &A);
    if (sz == 0) break;
    if (A0 < 0) A0 = A;
    offs.push_back(pos);
    pos += sz;
  }
  const int64_t hdr[2] = {(int64_t)offs.size(), (int64_t)(A0 < 0 ? 0 : A0)};
  fwrite(hdr, sizeof hdr, 1, stdout);
  std::vector<float> xyz(3 * (size_t)hdr[1]);
  for (int64_t off : offs) {
    int32_t step = 0;
    float time = 0.f, box[9] = {0};
    const int32_t st = gb::xtc::decode_frame(data, nbytes, off, A0, xyz.data(), &step, &time, box);
    fwrite(&st, 4, 1, stdout);
    fwrite(&step, 4, 1, stdout);
    fwrite(&time, 4, 1, stdout);
    fwrite(box, 4, 9, stdout);
    fwrite(xyz.data(), 4, xyz.size(), stdout);
  }
  return 0;
}
