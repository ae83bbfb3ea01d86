// Round-robin ("circle") pair schedule of the cyclic Jacobi and the row
// hand-over it implies when the pair slots are split over the CTAs of a
// cluster. Host and device code: the host side is exercised by the CPU tests.
#pragma once

#ifdef __CUDACC__
#define TSVD_HD __host__ __device__ __forceinline__
#else
#define TSVD_HD inline
#endif

namespace tsvd {

// Player at circle position `pos` (<= np-1) in round `t` (< np-1) of a
// round-robin over np players. Slot k of round t pairs positions k and
// np-1-k. From one round to the next every player at position j >= 2 moves to
// j-1, the player at 1 moves to np-1, position 0 stays.
TSVD_HD int circle_player(int pos, int t, int np) {
  if (pos == 0) return 0;
  int x = pos - 1 + t;
  if (x >= np - 1) x -= np - 1;
  return x + 1;
}

// Row hand-over after a round for the CTA that owns slots [s0, s0 + nloc)
// of P (P >= 2). top[i] / bot[i] name the buffers holding the rows of the
// players at positions s0 + i and np-1-(s0 + i). A CTA with s0 > 0 sends its
// first top row to the left neighbour, one with s0 + nloc < P its last bottom
// row to the right neighbour, and receives one row from each neighbour it
// has; the buffers of the rows it sent take the rows it receives.
// circle_arrivals gives the buffers the rows from the left (*dst_l) and right
// (*dst_r) neighbour go to (-1: none arrives); circle_next gives slot i's
// buffers in the next round. Both only read the current maps, so every slot
// can be renamed at once into a second pair of maps.
TSVD_HD void circle_arrivals(const int *top, const int *bot, int s0, int nloc, int P, int *dst_l,
                             int *dst_r) {
  const bool has_l = s0 > 0, has_r = s0 + nloc < P;
  int freed[2] = {-1, -1}, nfree = 0, used = 0;
  if (has_l) freed[nfree++] = top[0];
  if (has_r) freed[nfree++] = bot[nloc - 1];
  *dst_l = -1;
  *dst_r = -1;
  const int first = s0 == 0 ? 1 : 0;                  // slot 0's top never moves
  if (nloc - 1 >= first && has_r) *dst_r = freed[used++];  // last owned top: from the right
  if (s0 == 0) {
    if (nloc == 1) *dst_r = freed[used++];  // position 1 -> np-1 arrives from the right
  } else {
    *dst_l = freed[used++];  // first owned bottom: from the left
  }
}

TSVD_HD void circle_next(const int *top, const int *bot, int s0, int nloc, int P, int i,
                         int dst_l, int dst_r, int *ntop, int *nbot) {
  // tops: position j -> j - 1 (j >= 2), position P -> P - 1 from the bottom
  if (s0 + i == 0)
    *ntop = top[0];
  else if (i + 1 < nloc)
    *ntop = top[i + 1];
  else
    *ntop = (s0 + nloc < P) ? dst_r : bot[nloc - 1];
  // bottoms: position j -> j - 1, position 1 -> np - 1 (slot 0's bottom)
  if (i >= 1)
    *nbot = bot[i - 1];
  else if (s0 == 0)
    *nbot = nloc > 1 ? top[1] : dst_r;
  else
    *nbot = dst_l;
}

}  // namespace tsvd
