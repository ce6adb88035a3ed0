// Host check of the streaming kernel's dealing (mdtraj_gb300/csrc/
// stream_deal.cuh): for each line "frames grid warps splits" on stdin,
// replays every warp's unit sequence as the kernel walks it (deal_place for
// the first unit, deal_next after each) and checks that
//   * every unit in [0, frames * splits) is dealt exactly once;
//   * with one unit per frame, each CTA's local indices (fin_local_index of
//     the k-th frame of each warp) are exactly 0 .. n-1 for fin_slice_of's
//     n, fin_frame_of maps each back to the frame streamed there, the
//     refinement-list bases are the running sums of n, and no CTA holds more
//     frames than fin_max_frames (the shared-memory record slots).
// Prints "ok <cases>" or the first failure.
#include <cstdio>
#include <vector>

#include "../mdtraj_gb300/csrc/stream_deal.cuh"

using namespace gb;

static int check(int64_t F, int64_t grid, int warps, int64_t S) {
  const int64_t W = grid * warps, units = F * S;
  const Deal d = make_deal(units, W);
  std::vector<int> seen(units, 0);
  std::vector<int64_t> slot_frame;  // per CTA: local index -> frame
  std::vector<std::vector<int64_t>> ctas(grid);
  for (int64_t b = 0; b < grid; ++b) ctas[b].assign(fin_max_frames(F, grid, warps), -1);
  for (int64_t g = 0; g < W; ++g) {
    const int64_t b = g / warps;
    const int w = (int)(g % warps);
    int64_t k = 0;
    for (int64_t u = deal_place(g, d.full_units, d.part_shift, units); u < units;
         u = deal_next(u, W, d.full_units, d.part_shift, units), ++k) {
      if (u < 0) { printf("FAIL %lld %lld %d %lld: negative unit\n", (long long)F, (long long)grid, warps, (long long)S); return 1; }
      seen[u] += 1;
      if (S == 1) {
        const int64_t li = fin_local_index(k, w, d.full_rounds, d.part_shift, b, warps);
        if (li < 0 || li >= (int64_t)ctas[b].size() || ctas[b][li] != -1) {
          printf("FAIL %lld %lld %d 1: CTA %lld local index %lld out of range or taken\n", (long long)F,
                 (long long)grid, warps, (long long)b, (long long)li);
          return 1;
        }
        ctas[b][li] = u;
      }
    }
  }
  for (int64_t u = 0; u < units; ++u)
    if (seen[u] != 1) {
      printf("FAIL %lld %lld %d %lld: unit %lld dealt %d times\n", (long long)F, (long long)grid, warps, (long long)S,
             (long long)u, seen[u]);
      return 1;
    }
  if (S != 1) return 0;
  int64_t base = 0;
  for (int64_t b = 0; b < grid; ++b) {
    const FinSlice s = fin_slice_of(F, grid, b, warps);
    if (s.base != base) {
      printf("FAIL %lld %lld %d 1: CTA %lld base %lld, expected %lld\n", (long long)F, (long long)grid, warps,
             (long long)b, (long long)s.base, (long long)base);
      return 1;
    }
    base += s.n;
    for (int64_t i = 0; i < (int64_t)ctas[b].size(); ++i) {
      const bool in = i < s.n;
      if (in != (ctas[b][i] >= 0) || (in && fin_frame_of(s, i, grid, b, warps) != ctas[b][i])) {
        printf("FAIL %lld %lld %d 1: CTA %lld local index %lld\n", (long long)F, (long long)grid, warps, (long long)b,
               (long long)i);
        return 1;
      }
    }
  }
  if (base != F) {
    printf("FAIL %lld %lld %d 1: CTAs hold %lld frames\n", (long long)F, (long long)grid, warps, (long long)base);
    return 1;
  }
  return 0;
}

int main() {
  long long F, grid, S;
  int warps, n = 0;
  while (scanf("%lld %lld %d %lld", &F, &grid, &warps, &S) == 4) {
    if (check(F, grid, warps, S)) return 1;
    ++n;
  }
  printf("ok %d\n", n);
  return 0;
}
