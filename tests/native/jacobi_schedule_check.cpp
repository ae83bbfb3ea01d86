// Host check of the Jacobi kernel's row hand-over (circle_arrivals and
// circle_next): C CTAs,
// each owning a contiguous range of pair slots, pass rows through two
// mailboxes per round; after every round each owned slot must hold the two
// players circle_player assigns it, in distinct non-mailbox buffers.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "jacobi_sched.h"

using namespace tsvd;

int main() {
  int bad = 0, cases = 0;
  for (int np = 4; np <= 260; np += 2) {
    const int P = np / 2;
    for (int C = 1; C <= 16; ++C) {
      const int L = (P + C - 1) / C;
      if ((C - 1) * L >= P) continue;  // the kernel's launcher never picks this C
      ++cases;
      const int nbuf = 2 * L + 2, mbL = 2 * L, mbR = 2 * L + 1;
      std::vector<std::vector<int>> buf(C, std::vector<int>(nbuf, -1)), top(C), bot(C);
      for (int c = 0; c < C; ++c) {
        const int s0 = c * L, nloc = std::min(P, s0 + L) - s0;
        top[c].resize(nloc);
        bot[c].resize(nloc);
        for (int i = 0; i < nloc; ++i) {
          top[c][i] = 2 * i;
          bot[c][i] = 2 * i + 1;
          buf[c][2 * i] = s0 + i;
          buf[c][2 * i + 1] = np - 1 - (s0 + i);
        }
      }
      for (int t = 0; t < 3 * (np - 1) + 1; ++t) {
        const int tt = t % (np - 1);
        for (int c = 0; c < C; ++c) {
          const int s0 = c * L, nloc = (int)top[c].size();
          for (int i = 0; i < nloc; ++i) {
            const int k = s0 + i;
            if (buf[c][top[c][i]] != circle_player(k, tt, np) ||
                buf[c][bot[c][i]] != circle_player(np - 1 - k, tt, np)) {
              if (bad < 5)
                std::printf("np %d C %d round %d slot %d: holds %d/%d, schedule %d/%d\n", np, C, t,
                            k, buf[c][top[c][i]], buf[c][bot[c][i]], circle_player(k, tt, np),
                            circle_player(np - 1 - k, tt, np));
              ++bad;
            }
          }
        }
        std::vector<std::vector<int>> next = buf;  // the hand-over writes
        for (int c = 0; c < C; ++c) {
          const int s0 = c * L, nloc = (int)top[c].size();
          if (s0 > 0) next[c - 1][mbR] = buf[c][top[c][0]];
          if (s0 + nloc < P) next[c + 1][mbL] = buf[c][bot[c][nloc - 1]];
        }
        buf = next;
        for (int c = 0; c < C; ++c) {
          const int s0 = c * L, nloc = (int)top[c].size();
          int dl, dr;
          circle_arrivals(top[c].data(), bot[c].data(), s0, nloc, P, &dl, &dr);
          std::vector<int> nt(nloc), nb(nloc);
          for (int i = 0; i < nloc; ++i)
            circle_next(top[c].data(), bot[c].data(), s0, nloc, P, i, dl, dr, &nt[i], &nb[i]);
          top[c] = nt;
          bot[c] = nb;
          if (dl >= 0) buf[c][dl] = buf[c][mbL];
          if (dr >= 0) buf[c][dr] = buf[c][mbR];
          std::vector<int> seen(nbuf, 0);
          for (int i = 0; i < nloc; ++i)
            for (int b : {top[c][i], bot[c][i]}) {
              if (b < 0 || b >= 2 * L || seen[b]++) {
                if (bad < 5) std::printf("np %d C %d: buffer %d reused or out of range\n", np, C, b);
                ++bad;
              }
            }
        }
      }
    }
  }
  std::printf("cases %d mismatches %d\n", cases, bad);
  return bad != 0;
}
