// Halo finder (src/exshalos/find_halos.c:108-563) on sm_103a.
//
//  find_peaks   Count_Peaks/Find_Peaks (:108-156): strict 6-neighbour maxima,
//               compacted in row-major order.
//  sort_peaks   quickSort_peaks (:175-197) reproduced exactly, tie order
//               included.  Each Lomuto partition is computed in parallel:
//               elements <= pivot keep their order at their L-rank; an
//               element > pivot at relative position a moves along
//               a <- a + g(a) (g = number of > elements before the L with
//               rank a) until a >= nL; the one landing on nL swaps with the
//               pivot into the last slot.  Runs of equal g are crossed in one
//               step, so each element costs O(distinct g values crossed).
//               Large segments use all SMs per level; segments of at most
//               SORT_SMALL elements finish inside one block, one warp per
//               pending segment.
//  grow_halos   Grow_Halos (:215-379) with deterministic reservations: every
//               pending peak reserves the cells its exclusion-free growth
//               could read; peaks holding all their cells are grown exactly
//               (double running means in the reference's operation order,
//               no contraction) in the same round.  Halo numbers are assigned
//               afterwards in processing order.
//  halo_masses  Compute_Mass (:455-476): the taus stream is advanced to each
//               halo's draw by GF(2) jump matrices.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "halos.cuh"
#include "intdiv.cuh"
#include "scan.cuh"
#include "taus.cuh"

namespace exh {

// ------------------------------------------------------------------ shells
int build_shell_tables(Ctx& c, const BoxParams& b, int Ncells, ShellTable* t, cudaStream_t st) {
  const int T = b.nmin / 2;
  if (c.shell_ncells == Ncells && c.shell_nmin == b.nmin && c.buf[B_HALO2].p) {
    int* base = c.buf[B_HALO2].as<int>();
    t->gmax = c.shell_gmax;
    t->off_cap = base;
    t->off_all = base + c.shell_ncap;
    t->start_cap = t->off_all + c.shell_nall;
    t->start_all = t->start_cap + (t->gmax + 2);
    return EXH_OK;
  }
  c.shell_ncells = -1;
  const std::vector<int>& cis = cells_in_spheres();
  // last shell needed: the first r^2 whose cumulative count reaches Ncells
  long cum = 0;
  int gmax = -1;
  std::vector<long> hist;
  const int tmax = 64;
  hist.assign((size_t)3 * tmax * tmax + 1, 0);
  for (int i = -tmax; i <= tmax; i++)
    for (int j = -tmax; j <= tmax; j++)
      for (int k = -tmax; k <= tmax; k++) {
        const int d = i * i + j * j + k * k;
        if (d < (int)hist.size()) hist[d]++;
      }
  for (int g = 0; g < tmax * tmax; g++) {
    cum += hist[g];
    if (cum >= Ncells) { gmax = g; break; }
  }
  (void)cis;
  if (gmax < 0) {
    exh_set_error_msg("Ncells beyond the shell table", __FILE__, __LINE__);
    return EXH_E_RANGE;
  }
  t->gmax = gmax;
  const int r = (int)std::floor(std::sqrt((double)gmax)) + 1;
  std::vector<int> oc, oa, sc(gmax + 2, 0), sa(gmax + 2, 0);
  for (int g = 0; g <= gmax; g++) {
    sc[g] = (int)oc.size();
    sa[g] = (int)oa.size();
    const int tg = (int)std::floor(std::sqrt((double)g));
    for (int i = -tg; i <= tg; i++)
      for (int j = -tg; j <= tg; j++)
        for (int k = -tg; k <= tg; k++) {
          if (i * i + j * j + k * k != g) continue;
          const int packed = (i + 128) | ((j + 128) << 8) | ((k + 128) << 16);
          oa.push_back(packed);
          if (std::abs(i) <= T && std::abs(j) <= T && std::abs(k) <= T) oc.push_back(packed);
        }
  }
  sc[gmax + 1] = (int)oc.size();
  sa[gmax + 1] = (int)oa.size();
  (void)r;
  const size_t bytes = sizeof(int) * (oc.size() + oa.size() + 2 * (size_t)(gmax + 2));
  EXH_TRY(c.buf[B_HALO2].ensure(bytes));
  int* base = c.buf[B_HALO2].as<int>();
  t->off_cap = base;
  t->off_all = base + oc.size();
  t->start_cap = t->off_all + oa.size();
  t->start_all = t->start_cap + (gmax + 2);
  std::vector<int> host;
  host.reserve(bytes / 4);
  host.insert(host.end(), oc.begin(), oc.end());
  host.insert(host.end(), oa.begin(), oa.end());
  host.insert(host.end(), sc.begin(), sc.end());
  host.insert(host.end(), sa.begin(), sa.end());
  EXH_CUDA_TRY(cudaMemcpyAsync(base, host.data(), bytes, cudaMemcpyHostToDevice, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  c.shell_ncells = Ncells;
  c.shell_nmin = b.nmin;
  c.shell_gmax = gmax;
  c.shell_ncap = oc.size();
  c.shell_nall = oa.size();
  return EXH_OK;
}

__device__ __forceinline__ void unpack_off(int p, int& i, int& j, int& k) {
  i = (p & 0xff) - 128;
  j = ((p >> 8) & 0xff) - 128;
  k = ((p >> 16) & 0xff) - 128;
}

// ------------------------------------------------------------------ peaks
// Strict maximum against the six periodic neighbours (find_halos.c:108-156).
// The seven values of a cell are loaded before any comparison, so the loads
// are in flight together (a short-circuit chain would issue them one by one).
__device__ __forceinline__ void peak_load(const float* __restrict__ d, size_t cell, size_t ng, int n0, int n1,
                                          int n2, float (&a)[7]) {
  int i, j, k;
  cell_ijk(cell, ng, n1, n2, &i, &j, &k);
  const size_t s1 = n2, s0 = (size_t)n1 * n2;
  const size_t c = (size_t)i * s0 + (size_t)j * s1;
  a[0] = d[cell];
  a[1] = d[(size_t)exh_wrap(i, 1, n0) * s0 + (size_t)j * s1 + k];
  a[2] = d[(size_t)exh_wrap(i, -1, n0) * s0 + (size_t)j * s1 + k];
  a[3] = d[(size_t)i * s0 + (size_t)exh_wrap(j, 1, n1) * s1 + k];
  a[4] = d[(size_t)i * s0 + (size_t)exh_wrap(j, -1, n1) * s1 + k];
  a[5] = d[c + exh_wrap(k, 1, n2)];
  a[6] = d[c + exh_wrap(k, -1, n2)];
}
// The same for grids of fewer than 2^32 cells: (i, j, k) by two fast
// divisions and the six neighbours as 32-bit index offsets with the
// periodic wrap applied by a branch per axis (s0 = n1 n2, ng32 = n0 s0).
struct PeakGeom {
  FastDiv fd1, fd2;
  uint32_t n0, n1, n2, s0, ng32;
};
__device__ __forceinline__ void peak_load32(const float* __restrict__ d, uint32_t c, const PeakGeom& q,
                                            float (&a)[7]) {
  const uint32_t r = fd_div(c, q.fd2), k = c - r * q.n2;
  const uint32_t i = fd_div(r, q.fd1), j = r - i * q.n1;
  a[0] = d[c];
  a[1] = d[i + 1 == q.n0 ? c - (q.ng32 - q.s0) : c + q.s0];
  a[2] = d[i == 0 ? c + (q.ng32 - q.s0) : c - q.s0];
  a[3] = d[j + 1 == q.n1 ? c - (q.s0 - q.n2) : c + q.n2];
  a[4] = d[j == 0 ? c + (q.s0 - q.n2) : c - q.n2];
  a[5] = d[k + 1 == q.n2 ? c - (q.n2 - 1) : c + 1];
  a[6] = d[k == 0 ? c + (q.n2 - 1) : c - 1];
}
__device__ __forceinline__ bool peak_test(const float (&a)[7]) {
  return (a[0] > a[1]) & (a[0] > a[2]) & (a[0] > a[3]) & (a[0] > a[4]) & (a[0] > a[5]) & (a[0] > a[6]);
}

constexpr int PK_T = 256;          // cells per group: one count, eight mask words
constexpr int PK_U = 4;            // groups a block takes at once (their loads in flight together)
constexpr int PK_BLOCKS_PER_SM = 8;
constexpr int PK_MASK_BLOCKS_PER_SM = 5;   // resident blocks of k_peak_mask (its launch bound)

// one bit per cell (mask word w: cells 32 w .. 32 w + 31) and the peak count
// of every group of PK_T cells; blocks stride over runs of PK_U groups
__global__ void __launch_bounds__(PK_T, PK_MASK_BLOCKS_PER_SM)
k_peak_mask(const float* __restrict__ d, int n0, int n1, int n2, size_t ng, unsigned ngroups, PeakGeom q,
            unsigned* __restrict__ mask, unsigned* __restrict__ cnt) {
  const bool small = ng <= 0xffffffffull;
  __shared__ unsigned wc[PK_U][PK_T / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (unsigned g0 = blockIdx.x * PK_U; g0 < ngroups; g0 += gridDim.x * PK_U) {
    float a[PK_U][7];
    bool live[PK_U];
#pragma unroll
    for (int u = 0; u < PK_U; u++) {
      const size_t cell = (size_t)(g0 + u) * PK_T + threadIdx.x;
      live[u] = g0 + u < ngroups && cell < ng;
      if (live[u]) {
        if (small) peak_load32(d, (uint32_t)cell, q, a[u]);
        else peak_load(d, cell, ng, n0, n1, n2, a[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < PK_U; u++) {
      const unsigned m = __ballot_sync(0xffffffffu, live[u] && peak_test(a[u]));
      if (lane == 0 && g0 + u < ngroups) {
        mask[((size_t)(g0 + u) * PK_T >> 5) + w] = m;
        wc[u][w] = __popc(m);
      }
    }
    __syncthreads();
    if (threadIdx.x < PK_U && g0 + threadIdx.x < ngroups) {
      unsigned s = 0;
      for (int q = 0; q < PK_T / 32; q++) s += wc[threadIdx.x][q];
      cnt[g0 + threadIdx.x] = s;
    }
    __syncthreads();
  }
}

// peaks in row-major cell order: group offset + the peaks of the words
// before in the group + the lanes before in the word
__global__ void __launch_bounds__(PK_T)
k_peak_write(const float* __restrict__ d, size_t ng, unsigned ngroups, const unsigned* __restrict__ mask,
             const unsigned* __restrict__ off, float* __restrict__ key, unsigned* __restrict__ id) {
  __shared__ unsigned wo[PK_T / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (unsigned g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const size_t cell = (size_t)g * PK_T + threadIdx.x;
    const unsigned m = mask[cell >> 5];
    if (lane == 0) wo[w] = __popc(m);
    __syncthreads();
    unsigned before = 0;
    for (int q = 0; q < w; q++) before += wo[q];
    if (cell < ng && ((m >> lane) & 1u)) {
      const unsigned pos = off[g] + before + __popc(m & ((1u << lane) - 1u));
      key[pos] = d[cell];
      id[pos] = (unsigned)cell;
    }
    __syncthreads();
  }
}

// peaks the B_PEAKS buffer holds: its sets of keys and cell ids are laid out
// by the allocation's capacity, not the peak count, so buffer addresses
// (and the sort's captured graph) stay the same from one realisation to the
// next while the buffer does not grow
size_t peak_cap(const Ctx& c) { return c.buf[B_PEAKS].cap / ((sizeof(float) + sizeof(unsigned)) * 3); }

// B_SORT after find_peaks: the peak bitmask (one bit per cell), the peak
// count and the first peak (in cell order) of every group of PK_T cells.
// Only find_peaks writes the buffer, so it describes the peaks of the last
// grid searched, which are the peaks in use (a reused sort belongs to that
// grid too).
static void peak_mask_layout(Ctx& c, size_t ng, unsigned** mask, unsigned** cnt, unsigned** off) {
  const unsigned nb = exh_div_up(ng, PK_T);
  const size_t words = (size_t)nb * (PK_T / 32);
  *mask = c.buf[B_SORT].as<unsigned>();
  *cnt = *mask + words;
  *off = *cnt + nb;
}

int find_peaks(Ctx& c, const float* delta, const BoxParams& b, HaloDev* h, cudaStream_t st) {
  const size_t ng = b.ng;
  const unsigned nb = exh_div_up(ng, PK_T);
  const size_t words = (size_t)nb * (PK_T / 32);
  // scratch: mask words, block counts, block offsets, scan sums, total
  EXH_TRY(c.buf[B_SORT].ensure(sizeof(unsigned) * (words + 3 * (size_t)nb + 64)));
  unsigned *mask, *cnt, *off;
  peak_mask_layout(c, ng, &mask, &cnt, &off);
  unsigned* sums = off + nb;
  unsigned* total = sums + nb + 32;
  const unsigned grid = std::min<unsigned>(nb, EXH_NUM_SMS * PK_BLOCKS_PER_SM);
  const unsigned grid_m = std::min<unsigned>(exh_div_up(nb, PK_U), EXH_NUM_SMS * PK_MASK_BLOCKS_PER_SM);
  { KTimer kt(KC_PEAKS, st, 4.0 * ng + ng / 8.0);
  PeakGeom q;
  q.fd1 = make_fastdiv((uint32_t)b.nd[1]);
  q.fd2 = make_fastdiv((uint32_t)b.nd[2]);
  q.n0 = b.nd[0]; q.n1 = b.nd[1]; q.n2 = b.nd[2];
  q.s0 = q.n1 * q.n2;
  q.ng32 = (uint32_t)ng;            // used only while ng < 2^32
  k_peak_mask<<<grid_m, PK_T, 0, st>>>(delta, b.nd[0], b.nd[1], b.nd[2], ng, nb, q, mask, cnt); }
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  EXH_CUDA_TRY(exclusive_scan<unsigned>(cnt, off, nb, sums, total, st));
  unsigned np = 0;
  EXH_CUDA_TRY(cudaMemcpyAsync(&np, total, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  h->np = np;
  EXH_TRY(c.buf[B_PEAKS].ensure((sizeof(float) + sizeof(unsigned)) * std::max<size_t>(np, 1) * 3));
  const size_t cap = peak_cap(c);
  h->key = c.buf[B_PEAKS].as<float>();
  h->id = reinterpret_cast<unsigned*>(h->key + cap);
  { KTimer kt(KC_PEAKS, st, ng / 8.0 + 12.0 * np);
  k_peak_write<<<grid, PK_T, 0, st>>>(delta, ng, nb, mask, off, h->key, h->id); }
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

// ------------------------------------------------------------------ sort
constexpr int SORT_SMALL = 2048;     // segment size finished inside one block
constexpr int SORT_T = 512;
constexpr int CH_T = 256, CH_ITEMS = 8, CH = CH_T * CH_ITEMS;

struct Seg {
  int lo, hi;   // inclusive
  int buf;      // ping-pong buffer holding the segment
  int pad;
};

// Final position (relative) of the > element at relative position a.
// lam(q): number of <= elements before the q-th > element (nondecreasing);
// posl(r): relative position of the <= element of rank r, so that
// g(a) = posl(a) - a is the number of > elements before it.
template <typename LamT, typename PosT>
__device__ __forceinline__ int lomuto_g_dest(int a, int nL, int m, LamT lam, PosT posl) {
  while (a < nL) {
    const int c = posl(a) - a;                     // >= 1 for consistent input
    if (c <= 0) return nL;                         // never loop on inconsistent input
    const int bnd = c < m ? min(lam(c), nL) : nL;
    const int steps = (bnd - a + c - 1) / c;
    a += c * steps;
  }
  return a;
}

// per-chunk L counts
__global__ void k_qs_count(const float* __restrict__ key, const Seg* __restrict__ segs, const int* __restrict__ cseg,
                           const int* __restrict__ coff, const int* __restrict__ nchunks, int* __restrict__ cL) {
  const int ch = blockIdx.x;
  if (ch >= *nchunks) return;
  const Seg s = segs[cseg[ch]];
  const float pv = key[s.hi];
  const int start = s.lo + coff[ch], end = min(start + CH, s.hi);
  int n = 0;
  for (int p = start + threadIdx.x; p < end; p += CH_T) n += key[p] <= pv;
  __shared__ int ws[32];
  int tot;
  block_exclusive_scan<int>(n, ws, tot);
  if (threadIdx.x == 0) cL[ch] = tot;
}

__global__ void k_qs_seg_scan(const int* __restrict__ cfirst, const int* __restrict__ nseg, int* __restrict__ cL,
                              int* __restrict__ segNL) {
  const int sidx = blockIdx.x;
  if (sidx >= *nseg) return;
  const int c0 = cfirst[sidx], c1 = cfirst[sidx + 1];
  __shared__ int ws[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = c0; base < c1; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < c1 ? cL[i] : 0;
    int tot;
    const int ex = block_exclusive_scan<int>(v, ws, tot);
    if (i < c1) cL[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) segNL[sidx] = carry;
}

// L placement, lam, pivot (phase 1); the run end of every L rank (phase 3);
// > placement (phase 2).  chain[rank] = (posl(rank), run end): the position
// of the L element of that rank and the L count at the end of its run of L
// elements (min(lam(g), nL), or nL when no > element follows), so a step of
// the > chain is one 8-byte load.
template <int PHASE>
__global__ void __launch_bounds__(CH_T)
k_qs_place(const float* __restrict__ key, const unsigned* __restrict__ id, const Seg* __restrict__ segs,
           const int* __restrict__ cseg, const int* __restrict__ coff, const int* __restrict__ nchunks,
           const int* __restrict__ cLoff, const int* __restrict__ segNL, int* __restrict__ lam,
           int2* __restrict__ chain, float* __restrict__ okey, unsigned* __restrict__ oid, float* __restrict__ fkey,
           unsigned* __restrict__ fid, const int* __restrict__ jt) {
  const int ch = blockIdx.x;
  if (ch >= *nchunks) return;
  const int sidx = cseg[ch];
  const Seg s = segs[sidx];
  const float pv = key[s.hi];
  const int nL = segNL[sidx];
  const int start = s.lo + coff[ch], end = min(start + CH, s.hi);
  const int base = start + threadIdx.x * CH_ITEMS;
  const int m = (s.hi - s.lo) - nL;
  bool isL[CH_ITEMS];
  int n = 0;
#pragma unroll
  for (int q = 0; q < CH_ITEMS; q++) {
    const int p = base + q;
    isL[q] = p < end && key[p] <= pv;
    n += isL[q];
  }
  if (PHASE == 2) {
    // every > element follows its chain; the thread's chains advance in
    // lockstep so their loads overlap
    int a[CH_ITEMS];
    bool act[CH_ITEMS];
#pragma unroll
    for (int q = 0; q < CH_ITEMS; q++) {
      const int p = base + q;
      act[q] = p < end && !isL[q];
      a[q] = p - s.lo;
    }
    // a chain position a < nL is an L rank, so every load of the jump table
    // moves a chain JUMP_STEPS steps or to its end
    const int* js = jt + s.lo;
    for (int it = 0; it <= s.hi - s.lo; it++) {      // each load moves a chain up to four steps
      bool any = false;
#pragma unroll
      for (int q = 0; q < CH_ITEMS; q++) {
        if (act[q] && a[q] < nL) {
          const int nx = __ldg(&js[a[q]]);
          a[q] = nx > a[q] ? nx : nL;                   // never loop on inconsistent input
          any = true;
        }
      }
      if (!any) break;
    }
#pragma unroll
    for (int q = 0; q < CH_ITEMS; q++) {
      if (!act[q]) continue;
      const int p = base + q;
      const int dest = (a[q] >= nL) ? ((a[q] == nL) ? (s.hi - s.lo) : a[q]) : a[q];
      okey[s.lo + dest] = key[p];
      oid[s.lo + dest] = id[p];
    }
    return;
  }
  __shared__ int ws[32];
  int tot;
  int rank = block_exclusive_scan<int>(n, ws, tot) + cLoff[ch];
#pragma unroll
  for (int q = 0; q < CH_ITEMS; q++) {
    const int p = base + q;
    if (p >= end) break;
    const int rel = p - s.lo;
    if (isL[q]) {
      if (PHASE == 1) {
        okey[s.lo + rank] = key[p];
        oid[s.lo + rank] = id[p];
        chain[s.lo + rank].x = rel;
      } else {                                   // PHASE 3: run end of this rank
        const int c = rel - rank;                // > elements before it
        chain[s.lo + rank].y = c < m ? min(lam[s.lo + c], nL) : nL;
      }
      rank++;
    } else if (PHASE == 1) {
      lam[s.lo + (rel - rank)] = rank;
    }
  }
  if (PHASE == 1 && coff[ch] == 0 && threadIdx.x == 0) {
    okey[s.lo + nL] = key[s.hi];
    oid[s.lo + nL] = id[s.hi];
    fkey[s.lo + nL] = key[s.hi];
    fid[s.lo + nL] = id[s.hi];
  }
}

// One step of a > chain from relative position a < nL, from its chain entry.
__device__ __forceinline__ int chain_next(int a, int2 v, int nL) {
  const int c = v.x - a;
  if (c <= 0) return nL;                           // never loop on inconsistent input
  const int steps = (v.y - a + c - 1) / c;
  return a + c * max(steps, 1);
}

// Jump table over the L ranks of every segment of the level (chains never
// share a position, and the step depends on the position only): jo[r] =
// the position JUMP_STEPS steps after r, or the chain's end (>= nL) if it
// comes first.  Phase 2 then walks JUMP_STEPS steps per load.  The table is
// built in one pass: every rank follows its own chain for JUMP_STEPS
// dependent loads, all ranks at once.
constexpr int JUMP_STEPS = 8;

__global__ void __launch_bounds__(CH_T)
k_qs_jump(const Seg* __restrict__ segs, const int* __restrict__ cseg, const int* __restrict__ coff,
          const int* __restrict__ nchunks, const int* __restrict__ segNL, const int2* __restrict__ chain,
          int* __restrict__ jo) {
  const int ch = blockIdx.x;
  if (ch >= *nchunks) return;
  const int sidx = cseg[ch];
  const Seg s = segs[sidx];
  const int nL = segNL[sidx];
  const int r0 = coff[ch], r1 = min(min(r0 + CH, s.hi - s.lo), nL);
  const int2* cs = chain + s.lo;
  constexpr int PER = CH / CH_T;                   // ranks per thread, followed together
  int a[PER];
#pragma unroll
  for (int q = 0; q < PER; q++) a[q] = r0 + threadIdx.x + q * CH_T;
#pragma unroll
  for (int st = 0; st < JUMP_STEPS; st++)
#pragma unroll
    for (int q = 0; q < PER; q++)
      if (a[q] < nL && r0 + threadIdx.x + q * CH_T < r1) a[q] = chain_next(a[q], __ldg(&cs[a[q]]), nL);
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int r = r0 + threadIdx.x + q * CH_T;
    if (r < r1) jo[s.lo + r] = a[q];
  }
}

// level bookkeeping on the device: counters of the level loop
struct SortCtl {
  int nseg, nch, nnext, nsmall, nsingle, err;
  int iters;                   // iterations of the graph's level loop
  int maxseg;                  // largest segment of the current level
  unsigned long long elems;    // elements partitioned by the level kernels (timing)
};

// Once every large segment holds at most MID_MAX elements, one block per
// segment finishes its levels (k_qs_mid) instead of a launch sequence per
// level: the last levels have few segments and take tens of microseconds
// each as a level of kernels.  (box_256: 16384 and 8192 sort alike, 32768
// about 0.1 ms slower, 65536 0.6 ms slower: one block then runs a long chain
// of levels.)
constexpr int MID_MAX = 16384;

struct SortBufs {
  float* kb[2];
  unsigned* ib[2];
};

// children of every partitioned segment: large ones to the next level,
// 2..SORT_SMALL elements to the block sort, single elements to the copy list
__global__ void k_qs_children(const Seg* __restrict__ segs, const int* __restrict__ segNL, SortCtl* ctl,
                              Seg* __restrict__ next, Seg* __restrict__ small, int2* __restrict__ single, int cap_next,
                              int cap_small) {
  const int sidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (sidx >= ctl->nseg) return;
  const Seg sg = segs[sidx];
  const int nL = segNL[sidx];
  const int nb = sg.buf ^ 1;
  const Seg ch[2] = {{sg.lo, sg.lo + nL - 1, nb, 0}, {sg.lo + nL + 1, sg.hi, nb, 0}};
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int len = ch[q].hi - ch[q].lo + 1;
    if (len > SORT_SMALL) {
      const int i = atomicAdd(&ctl->nnext, 1);
      if (i < cap_next) next[i] = ch[q]; else atomicExch(&ctl->err, 1);
    } else if (len >= 2) {
      const int i = atomicAdd(&ctl->nsmall, 1);
      if (i < cap_small) small[i] = ch[q]; else atomicExch(&ctl->err, 1);
    } else if (len == 1) {
      const int i = atomicAdd(&ctl->nsingle, 1);
      if (i < cap_small) single[i] = make_int2(ch[q].lo, nb); else atomicExch(&ctl->err, 1);
    }
  }
}

// next level's segment list and chunk tables (one block).  Inside the level
// loop's graph (cond_on), the last level of the loop body also decides
// whether the loop goes on: while large segments remain, no list
// overflowed, and at most SORT_ITERS_PER_LAUNCH iterations per launch (the
// host then launches the graph again).
constexpr int QS_CHUNK_T = 1024;
constexpr int SORT_ITERS_PER_LAUNCH = 64;
__global__ void __launch_bounds__(QS_CHUNK_T)
k_qs_chunks(SortCtl* ctl, const Seg* __restrict__ next, Seg* __restrict__ segs, int* __restrict__ cfirst,
            int* __restrict__ cseg, int* __restrict__ coff, int cap_chunks, cudaGraphConditionalHandle cond,
            int cond_on) {
  __shared__ int ws[32];
  __shared__ int carry, smax;
  const int nseg = ctl->nnext;
  if (threadIdx.x == 0) { carry = 0; smax = 0; }
  __syncthreads();
  for (int base = 0; base < nseg; base += QS_CHUNK_T) {
    const int i = base + threadIdx.x;
    Seg sg{0, 0, 0, 0};
    int n = 0;
    if (i < nseg) {
      sg = next[i];
      n = (sg.hi - sg.lo + CH - 1) / CH;        // chunks over the elements before the pivot
      segs[i] = sg;
      atomicAdd(&ctl->elems, (unsigned long long)(sg.hi - sg.lo + 1));
      atomicMax(&smax, sg.hi - sg.lo + 1);
    }
    int tot;
    const int ex = block_exclusive_scan<int>(n, ws, tot) + carry;
    if (i < nseg) cfirst[i] = ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) cfirst[nseg] = carry;
  __syncthreads();
  // chunk table: every chunk finds its segment by a binary search of the
  // segments' first chunks
  const int nch = min(carry, cap_chunks);
  for (int c = threadIdx.x; c < nch; c += blockDim.x) {
    int lo = 0, hi = nseg;                        // last segment whose first chunk is <= c
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (cfirst[mid] <= c) lo = mid; else hi = mid;
    }
    cseg[c] = lo;
    coff[c] = (c - cfirst[lo]) * CH;
  }
  if (threadIdx.x == 0) {
    if (carry > cap_chunks) ctl->err = 1;
    ctl->nseg = nseg;
    ctl->nch = min(carry, cap_chunks);
    ctl->nnext = 0;
    ctl->maxseg = smax;
    if (cond_on) {
      const int it = ++ctl->iters;
      cudaGraphSetConditional(cond, (nseg > 0 && smax > MID_MAX && ctl->err == 0 && it % SORT_ITERS_PER_LAUNCH != 0)
                                        ? 1u : 0u);
    }
  }
}

// The last levels of the large segments (each at most MID_MAX elements), one
// block per segment: every level partitions all of the block's pending
// sub-segments (more than SORT_SMALL elements) at once, as k_qs_place does
// (Lomuto: L elements to the front in order, pivot after them, > elements
// along their chains), in the ping-pong buffers and with the lam / posl
// tables in global memory at the segment's positions.  The sub-segments
// are processed as one concatenated index space in rounds of MID_T x MID_IT
// elements: one block scan per round gives the L ranks (minus the count
// before each sub-segment's first element).  Pivots go to their final
// places; children of at most SORT_SMALL elements go to the block sort's
// list, single elements to the copy list.  At most n levels.
constexpr int MID_T = 1024;
constexpr int MID_IT = 4;
constexpr int MID_PEND = 32;          // > MID_MAX / (SORT_SMALL + 1) pending sub-segments
__global__ void __launch_bounds__(MID_T)
k_qs_mid(const Seg* __restrict__ segs, SortCtl* ctl, SortBufs b, int* __restrict__ lam, int* __restrict__ posl,
         float* __restrict__ fkey, unsigned* __restrict__ fid, Seg* __restrict__ small, int2* __restrict__ single,
         int cap_small) {
  __shared__ int cur[2 * MID_PEND], nxt[4 * MID_PEND], pre[MID_PEND + 1], sbase[2 * MID_PEND];
  __shared__ int ncur;
  __shared__ int ws[32];
  const Seg sg = segs[blockIdx.x];
  int cb = sg.buf;
  if (threadIdx.x == 0) { cur[0] = sg.lo; cur[1] = sg.hi; ncur = 1; }
  __syncthreads();
  for (int level = 0; level <= sg.hi - sg.lo && ncur > 0; level++) {
    const int nc = ncur;
    const float* key = b.kb[cb];
    const unsigned* id = b.ib[cb];
    float* okey = b.kb[cb ^ 1];
    unsigned* oid = b.ib[cb ^ 1];
    if (threadIdx.x < 32) {                       // prefix of the pending sizes (nc <= MID_PEND)
      const int lane = threadIdx.x;
      int v = lane < nc ? cur[2 * lane + 1] - cur[2 * lane] + 1 : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
      }
      pre[lane + 1] = v;
      if (lane == 0) pre[0] = 0;
    }
    __syncthreads();
    const int total = pre[nc];
    // pass 1: L flags, L ranks, L elements in place, lam and posl
    int carry = 0;
    for (int rb = 0; rb < total; rb += MID_T * MID_IT) {
      const int i0 = rb + threadIdx.x * MID_IT;
      int q = 0;
      {
        int hi = nc;                              // last q with pre[q] <= i0
        while (hi - q > 1) {
          const int mid = (q + hi) >> 1;
          if (pre[mid] <= i0) q = mid; else hi = mid;
        }
      }
      int sq[MID_IT], pp[MID_IT];
      bool isL[MID_IT];
      int c = 0;
#pragma unroll
      for (int u = 0; u < MID_IT; u++) {
        const int i = i0 + u;
        while (q + 1 < nc && pre[q + 1] <= i) q++;
        sq[u] = -1;
        pp[u] = 0;
        isL[u] = false;
        if (i < total) {
          const int p = cur[2 * q] + (i - pre[q]), hi = cur[2 * q + 1];
          sq[u] = q;
          pp[u] = p;
          isL[u] = p < hi && key[p] <= key[hi];
        }
        c += isL[u];
      }
      int tot;
      const int r0 = block_exclusive_scan<int>(c, ws, tot) + carry;
      int r = r0;
#pragma unroll
      for (int u = 0; u < MID_IT; u++) {
        const int q2 = sq[u];
        if (q2 >= 0) {
          if (pp[u] == cur[2 * q2]) sbase[2 * q2] = r;
          if (pp[u] == cur[2 * q2 + 1]) sbase[2 * q2 + 1] = r;
        }
        r += isL[u];
      }
      __syncthreads();
      r = r0;
#pragma unroll
      for (int u = 0; u < MID_IT; u++) {
        const int q2 = sq[u];
        if (q2 >= 0 && pp[u] < cur[2 * q2 + 1]) {
          const int lo = cur[2 * q2], p = pp[u], rel = r - sbase[2 * q2];
          if (isL[u]) {
            okey[lo + rel] = key[p];
            oid[lo + rel] = id[p];
            posl[lo + rel] = p - lo;
          } else {
            lam[lo + (p - lo - rel)] = rel;
          }
        }
        r += isL[u];
      }
      carry += tot;
      __syncthreads();
    }
    // pass 2: the > elements along their chains, pivots to their final places
    for (int rb = 0; rb < total; rb += MID_T * MID_IT) {
      const int i0 = rb + threadIdx.x * MID_IT;
      int q = 0;
      {
        int hi = nc;
        while (hi - q > 1) {
          const int mid = (q + hi) >> 1;
          if (pre[mid] <= i0) q = mid; else hi = mid;
        }
      }
#pragma unroll
      for (int u = 0; u < MID_IT; u++) {
        const int i = i0 + u;
        while (q + 1 < nc && pre[q + 1] <= i) q++;
        if (i >= total) continue;
        const int lo = cur[2 * q], hi = cur[2 * q + 1], p = lo + (i - pre[q]);
        const int nL = sbase[2 * q + 1] - sbase[2 * q];
        if (p == hi) {
          okey[lo + nL] = key[hi];
          oid[lo + nL] = id[hi];
          fkey[lo + nL] = key[hi];
          fid[lo + nL] = id[hi];
        } else if (!(key[p] <= key[hi])) {
          const int* ls = lam + lo;
          const int* ps = posl + lo;
          const int a = lomuto_g_dest(p - lo, nL, (hi - lo) - nL, [ls](int k) { return ls[k]; },
                                      [ps](int k) { return ps[k]; });
          const int dest = (a == nL) ? hi - lo : a;
          okey[lo + dest] = key[p];
          oid[lo + dest] = id[p];
        }
      }
    }
    if (threadIdx.x < nc) {
      const int q = threadIdx.x, lo = cur[2 * q], hi = cur[2 * q + 1];
      const int nL = sbase[2 * q + 1] - sbase[2 * q];
      nxt[4 * q + 0] = lo;
      nxt[4 * q + 1] = lo + nL - 1;
      nxt[4 * q + 2] = lo + nL + 1;
      nxt[4 * q + 3] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int k = 0;
      for (int q = 0; q < 2 * nc; q++) {
        const int clo = nxt[2 * q], chi = nxt[2 * q + 1], len = chi - clo + 1;
        if (len > SORT_SMALL) {
          if (k < MID_PEND) { cur[2 * k] = clo; cur[2 * k + 1] = chi; k++; }
          else atomicExch(&ctl->err, 1);
        } else if (len >= 2) {
          const int j = atomicAdd(&ctl->nsmall, 1);
          if (j < cap_small) small[j] = Seg{clo, chi, cb ^ 1, 0}; else atomicExch(&ctl->err, 1);
        } else if (len == 1) {
          const int j = atomicAdd(&ctl->nsingle, 1);
          if (j < cap_small) single[j] = make_int2(clo, cb ^ 1); else atomicExch(&ctl->err, 1);
        }
      }
      ncur = k;
    }
    cb ^= 1;
    __syncthreads();
  }
  if (ncur > 0 && threadIdx.x == 0) atomicExch(&ctl->err, 1);
}

// copy finished single elements into the final arrays
__global__ void k_qs_copy_single(const int2* __restrict__ single, const SortCtl* ctl, SortBufs b,
                                 float* __restrict__ fkey, unsigned* __restrict__ fid) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ctl->nsingle) return;
  const int2 e = single[t];
  fkey[e.x] = b.kb[e.y][e.x];
  fid[e.x] = b.ib[e.y][e.x];
}

struct SmallSortBuffers {
  float* kb[2];
  unsigned* ib[2];
};

// Sub-segments of at most SORT_TINY elements are finished by one warp, one
// element per lane, with the literal Lomuto quicksort's result
// (find_halos.c:175-197: pivot at hi, keys <= pivot to the front in their
// order, then both sides).  A quicksort leaves distinct keys in ascending
// order whatever its pivots, so a pending sub-segment without two equal keys
// is finished at once (each lane's place is the number of smaller keys);
// the others partition, all at once per level: each is a run of lanes
// [a, b] (pivot in lane b), L ranks come from the warp's ballot, and a >
// element's place follows the same chain as in k_qs_place, with posl(r) (the
// r-th L lane) and lam(c) (L lanes before the c-th > lane) read off the two
// ballots.  At most 31 levels.
constexpr int SORT_TINY = 32;

// position of the n-th (0-based) set bit of m (m has more than n set bits)
__device__ __forceinline__ int nth_set(unsigned m, int n) {
  int pos = 0;
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) {
    const int c = __popc(m & ((1u << w) - 1u));
    if (n >= c) {
      n -= c;
      m >>= w;
      pos += w;
    }
  }
  return pos;
}

__device__ __forceinline__ void warp_tiny_sort(float* ka, unsigned* ia, float* kb, unsigned* ib, int lo, int hi,
                                               int lane) {
  constexpr unsigned FULL = 0xffffffffu;
  const int s = hi - lo + 1;                       // 2 .. SORT_TINY
  const bool act = lane < s;
  float k = act ? ka[lo + lane] : 0.f;
  unsigned id = act ? ia[lo + lane] : 0u;
  unsigned start = 1u;                             // lanes that begin a sub-segment
  unsigned pend = s >= 2 ? 1u : 0u;                // sub-segments (by first lane) still to partition
  while (pend) {
    const int a = 31 - __clz(start & ((2u << lane) - 1u));
    const unsigned above = start & ~((2u << lane) - 1u);
    const int b = (above ? __ffs(above) - 1 : s) - 1;
    const bool inpend = act && ((pend >> a) & 1u);
    // equal keys (-0 and +0 compare equal) within the pending sub-segment;
    // lanes outside the segment carry distinct NaN patterns
    const unsigned ab = ((2u << b) - 1u) & ~((1u << a) - 1u);       // lanes a .. b
    const unsigned same = __match_any_sync(FULL, act ? __float_as_uint(k == 0.f ? 0.f : k) : 0x7fc00000u + lane);
    const unsigned tiem = __ballot_sync(FULL, inpend && __popc(same & ab) > 1);
    const bool ranked = inpend && (tiem & ab) == 0u;
    int dest = lane;
    if (__any_sync(FULL, ranked)) {
      int rk = 0;
      for (int j = 0; j < 32; j++) {
        const float kj = __shfl_sync(FULL, k, j);
        rk += (j >= a && j <= b && kj < k) ? 1 : 0;
      }
      if (ranked) dest = a + rk;
    }
    const bool lom = inpend && !ranked;
    const float pv = __shfl_sync(FULL, k, b & 31);
    const bool isL = lom && lane < b && k <= pv;
    const bool isG = lom && lane < b && !(k <= pv);
    const unsigned Lm = __ballot_sync(FULL, isL), Gm = __ballot_sync(FULL, isG);
    unsigned add_start = 0u, add_pend = 0u;
    if (lom) {
      const unsigned seg = ((1u << b) - 1u) & ~((1u << a) - 1u);
      const int nL = __popc(Lm & seg), m = (b - a) - nL;
      if (isL) {
        dest = a + __popc(Lm & seg & ((1u << lane) - 1u));
      } else if (lane == b) {
        dest = a + nL;
      } else {
        const unsigned Lr = (Lm & seg) >> a, Gr = (Gm & seg) >> a;
        const int g = lomuto_g_dest(lane - a, nL, m, [Gr](int c) { return nth_set(Gr, c) - c; },
                                    [Lr](int r) { return nth_set(Lr, r); });
        dest = a + (g == nL ? b - a : g);
      }
      if (lane == a) {
        add_start = 1u << (a + nL);
        if (a + nL + 1 <= b) add_start |= 1u << (a + nL + 1);
        if (nL >= 2) add_pend |= 1u << a;
        if (m >= 2) add_pend |= 1u << (a + nL + 1);
      }
    }
    if (act) { kb[lo + dest] = k; ib[lo + dest] = id; }
    __syncwarp();
    if (act) { k = kb[lo + lane]; id = ib[lo + lane]; }
    __syncwarp();
    start |= __reduce_or_sync(FULL, add_start);
    pend = __reduce_or_sync(FULL, add_pend);
  }
  if (act) { ka[lo + lane] = k; ia[lo + lane] = id; }
}

// One block sorts one segment of at most SORT_SMALL elements, level by
// level.  Each level partitions every pending sub-segment (more than
// SORT_TINY elements) at once with the whole block (Lomuto, as k_qs_place):
// thread t owns positions IT t .. IT t + IT - 1; one block scan of the L
// flags over all positions gives every L element its rank (the scan value
// minus the value at its sub-segment's first position), and the > elements
// follow their chains.  The pending list stays ordered by position, so a
// position finds its sub-segment by a binary search of the list.  Children
// of at most SORT_TINY elements go to the warp sort.  No locks and no waits
// other than block barriers; at most n levels.
__global__ void __launch_bounds__(SORT_T)
k_qs_small(const Seg* __restrict__ segs, int nseg, SmallSortBuffers bufs, float* __restrict__ fkey,
           unsigned* __restrict__ fid, int* __restrict__ err) {
  constexpr int IT = SORT_SMALL / SORT_T;
  extern __shared__ unsigned char sm_raw[];
  float* ka = reinterpret_cast<float*>(sm_raw);
  unsigned* ia = reinterpret_cast<unsigned*>(ka + SORT_SMALL);
  float* kb = reinterpret_cast<float*>(ia + SORT_SMALL);
  unsigned* ib = reinterpret_cast<unsigned*>(kb + SORT_SMALL);
  int* lam = reinterpret_cast<int*>(ib + SORT_SMALL);
  int* posl = lam + SORT_SMALL;
  // pending sub-segments have more than SORT_TINY elements: at most
  // SORT_SMALL / (SORT_TINY + 1) of them; tiny ones at most SORT_SMALL / 2
  constexpr int PEND = 2 * (SORT_SMALL / (SORT_TINY + 1) + 1);
  static_assert(2 * PEND + 4 * PEND + 2 * PEND + SORT_SMALL <= 3 * SORT_SMALL, "lists fit the allocation");
  int* cur = posl + SORT_SMALL;             // pending (lo, hi) pairs of this level, by position
  int* nxt = cur + 2 * PEND;                // two child slots per pending segment
  int* sbase = nxt + 4 * PEND;              // L flags before each pending segment's first / last position
  int* tiny = sbase + 2 * PEND;             // (lo, hi) pairs finished by one warp each
  __shared__ int ncur, ntiny;
  __shared__ int ws[32];
  if (blockIdx.x >= nseg) return;
  const Seg sg = segs[blockIdx.x];
  const int n = sg.hi - sg.lo + 1;
  const float* sk = bufs.kb[sg.buf] + sg.lo;
  const unsigned* si = bufs.ib[sg.buf] + sg.lo;
  for (int t = threadIdx.x; t < n; t += blockDim.x) { ka[t] = sk[t]; ia[t] = si[t]; }
  if (threadIdx.x == 0) {
    ncur = 0;
    ntiny = 0;
    if (n > SORT_TINY) { cur[0] = 0; cur[1] = n - 1; ncur = 1; }
    else if (n >= 2) { tiny[0] = 0; tiny[1] = n - 1; ntiny = 1; }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int base = threadIdx.x * IT;
  for (int level = 0; level <= n && ncur > 0; level++) {
    const int nc = ncur;
    // sub-segment of each owned position (-1: none pending) and its L flag
    int sq[IT];
    bool isL[IT];
    int c = 0;
    int q = 0;
    {
      int qh = nc;                              // first q whose last position is >= base
      while (q < qh) {
        const int mid = (q + qh) >> 1;
        if (cur[2 * mid + 1] < base) q = mid + 1; else qh = mid;
      }
    }
#pragma unroll
    for (int u = 0; u < IT; u++) {
      const int p = base + u;
      while (q < nc && cur[2 * q + 1] < p) q++;
      const bool in = p < n && q < nc && cur[2 * q] <= p;
      sq[u] = in ? q : -1;
      isL[u] = in && p < cur[2 * q + 1] && ka[p] <= ka[cur[2 * q + 1]];
      c += isL[u];
    }
    int tot;
    const int r0 = block_exclusive_scan<int>(c, ws, tot);
    {
      int r = r0;
#pragma unroll
      for (int u = 0; u < IT; u++) {
        const int p = base + u, q = sq[u];
        if (q >= 0) {
          if (p == cur[2 * q]) sbase[2 * q] = r;
          if (p == cur[2 * q + 1]) sbase[2 * q + 1] = r;
        }
        r += isL[u];
      }
    }
    __syncthreads();
    // L elements to the front in order, lam and posl
    {
      int r = r0;
#pragma unroll
      for (int u = 0; u < IT; u++) {
        const int p = base + u, q = sq[u];
        if (q >= 0 && p < cur[2 * q + 1]) {
          const int lo = cur[2 * q], rel = r - sbase[2 * q];
          if (isL[u]) { kb[lo + rel] = ka[p]; ib[lo + rel] = ia[p]; posl[lo + rel] = p - lo; }
          else lam[lo + (p - lo - rel)] = rel;
        }
        r += isL[u];
      }
    }
    __syncthreads();
    // > elements along their chains, pivots after the L elements
#pragma unroll
    for (int u = 0; u < IT; u++) {
      const int p = base + u, q = sq[u];
      if (q < 0) continue;
      const int lo = cur[2 * q], hi = cur[2 * q + 1];
      const int nL = sbase[2 * q + 1] - sbase[2 * q];
      if (p == hi) {
        kb[lo + nL] = ka[p];
        ib[lo + nL] = ia[p];
      } else if (!isL[u]) {
        const int* ls = lam + lo;
        const int* ps = posl + lo;
        const int a = lomuto_g_dest(p - lo, nL, (hi - lo) - nL, [ls](int i) { return ls[i]; },
                                    [ps](int i) { return ps[i]; });
        const int dest = (a == nL) ? hi - lo : a;
        kb[lo + dest] = ka[p];
        ib[lo + dest] = ia[p];
      }
    }
    if (threadIdx.x < nc) {
      const int q = threadIdx.x, lo = cur[2 * q], hi = cur[2 * q + 1];
      const int nL = sbase[2 * q + 1] - sbase[2 * q], m = hi - lo - nL;
      nxt[4 * q + 0] = nL >= 2 ? lo : -1;
      nxt[4 * q + 1] = lo + nL - 1;
      nxt[4 * q + 2] = m >= 2 ? lo + nL + 1 : -1;
      nxt[4 * q + 3] = hi;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < IT; u++) {
      const int p = base + u;
      if (sq[u] >= 0) { ka[p] = kb[p]; ia[p] = ib[p]; }
    }
    {
      // children in slot order (left, right of each pending segment): large
      // ones to the next level, the others to the tiny list; one thread per
      // slot, places by a block scan of packed (large << 16 | tiny) counts
      const int nt0 = ntiny;
      const int q = threadIdx.x;
      int clo = -1, chi = -1, cnt = 0;
      if (q < 2 * nc) {
        clo = nxt[2 * q];
        chi = nxt[2 * q + 1];
        if (clo >= 0) cnt = (chi - clo + 1 > SORT_TINY) ? (1 << 16) : 1;
      }
      int ctot;
      const int ex = block_exclusive_scan<int>(cnt, ws, ctot);
      if (cnt == (1 << 16)) { cur[2 * (ex >> 16)] = clo; cur[2 * (ex >> 16) + 1] = chi; }
      else if (cnt == 1) { tiny[2 * (nt0 + (ex & 0xffff))] = clo; tiny[2 * (nt0 + (ex & 0xffff)) + 1] = chi; }
      __syncthreads();
      if (threadIdx.x == 0) {
        ncur = ctot >> 16;
        ntiny = nt0 + (ctot & 0xffff);
      }
    }
    __syncthreads();
  }
  if (ncur > 0 && threadIdx.x == 0) atomicExch(err, 1);
  for (int q = w; q < ntiny; q += nw) warp_tiny_sort(ka, ia, kb, ib, tiny[2 * q], tiny[2 * q + 1], lane);
  __syncthreads();
  for (int t = threadIdx.x; t < n; t += blockDim.x) { fkey[sg.lo + t] = ka[t]; fid[sg.lo + t] = ia[t]; }
}
int sort_peaks(Ctx& c, HaloDev* h, cudaStream_t st) {
  const int np = (int)h->np;
  const size_t cap = peak_cap(c);          // find_peaks laid the keys out by this capacity
  float* k0 = h->key;
  unsigned* i0 = h->id;
  float* k1 = reinterpret_cast<float*>(i0 + cap);
  unsigned* i1 = reinterpret_cast<unsigned*>(k1 + cap);
  // final arrays live in B_PEAKS2
  EXH_TRY(c.buf[B_PEAKS2].ensure((sizeof(float) + sizeof(unsigned)) * cap + sizeof(int) * (cap + 1) +
                                  sizeof(int2) * cap + sizeof(int) * cap + 16));
  float* fk = c.buf[B_PEAKS2].as<float>();
  unsigned* fi = reinterpret_cast<unsigned*>(fk + cap);
  int* lam = reinterpret_cast<int*>(fi + cap);
  int2* chain = reinterpret_cast<int2*>(lam + cap + (cap & 1));     // 8-byte aligned
  int* j2 = reinterpret_cast<int*>(chain + cap);                   // jump table of the > chains
  if (np <= 1) {
    if (np == 1) {
      EXH_CUDA_TRY(cudaMemcpyAsync(fk, k0, sizeof(float), cudaMemcpyDeviceToDevice, st));
      EXH_CUDA_TRY(cudaMemcpyAsync(fi, i0, sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
    }
    h->key = fk;
    h->id = fi;
    return EXH_OK;
  }
  float* kb[2] = {k0, k1};
  unsigned* ib[2] = {i0, i1};
  // device-side level loop: segment lists, chunk tables and counters live
  // on the device, sized by the capacity
  const int ncap = (int)std::min<size_t>(cap, (size_t)1 << 30);
  const int max_segs = ncap / SORT_SMALL + 8;
  const int max_chunks = ncap / CH + max_segs + 8;
  const int cap_small = ncap / 2 + 8;
  const size_t need = sizeof(SortCtl) + sizeof(Seg) * (2 * (size_t)max_segs + cap_small) +
                      sizeof(int2) * (size_t)cap_small +
                      sizeof(int) * (3 * (size_t)max_chunks + 2 * (size_t)max_segs + 8) + 64;
  EXH_TRY(c.buf[B_SCRATCH].ensure(need));
  SortCtl* ctl = c.buf[B_SCRATCH].as<SortCtl>();
  Seg* d_segs = reinterpret_cast<Seg*>(ctl + 1);
  Seg* d_next = d_segs + max_segs;
  Seg* d_small = d_next + max_segs;
  int2* d_single = reinterpret_cast<int2*>(d_small + cap_small);
  int* d_cseg = reinterpret_cast<int*>(d_single + cap_small);
  int* d_coff = d_cseg + max_chunks;
  int* d_cL = d_coff + max_chunks;
  int* d_cfirst = d_cL + max_chunks;
  int* d_nl = d_cfirst + max_segs + 1;
  SortCtl h0{};
  const Seg whole{0, np - 1, 0, 0};
  if (np > SORT_SMALL) h0.nnext = 1; else h0.nsmall = 1;
  EXH_TRY(upload_small(np > SORT_SMALL ? d_next : d_small, &whole, sizeof(Seg), st));
  EXH_TRY(upload_small(ctl, &h0, sizeof(SortCtl), st));
  SortCtl hc = h0;
  // one level: the large segments of buffer `buf` are partitioned into the
  // other buffer (or, finished, into the final arrays)
  auto level = [&](int buf, cudaStream_t s, cudaGraphConditionalHandle cond, int cond_on) -> int {
    k_qs_count<<<max_chunks, CH_T, 0, s>>>(kb[buf], d_segs, d_cseg, d_coff, &ctl->nch, d_cL);
    k_qs_seg_scan<<<max_segs, 256, 0, s>>>(d_cfirst, &ctl->nseg, d_cL, d_nl);
    k_qs_place<1><<<max_chunks, CH_T, 0, s>>>(kb[buf], ib[buf], d_segs, d_cseg, d_coff, &ctl->nch, d_cL, d_nl, lam,
                                              chain, kb[buf ^ 1], ib[buf ^ 1], fk, fi, j2);
    k_qs_place<3><<<max_chunks, CH_T, 0, s>>>(kb[buf], ib[buf], d_segs, d_cseg, d_coff, &ctl->nch, d_cL, d_nl, lam,
                                              chain, kb[buf ^ 1], ib[buf ^ 1], fk, fi, j2);
    k_qs_jump<<<max_chunks, CH_T, 0, s>>>(d_segs, d_cseg, d_coff, &ctl->nch, d_nl, chain, j2);
    k_qs_place<2><<<max_chunks, CH_T, 0, s>>>(kb[buf], ib[buf], d_segs, d_cseg, d_coff, &ctl->nch, d_cL, d_nl, lam,
                                              chain, kb[buf ^ 1], ib[buf ^ 1], fk, fi, j2);
    k_qs_children<<<exh_div_up(max_segs, 128), 128, 0, s>>>(d_segs, d_nl, ctl, d_next, d_small, d_single, max_segs,
                                                            cap_small);
    k_qs_chunks<<<1, QS_CHUNK_T, 0, s>>>(ctl, d_next, d_segs, d_cfirst, d_cseg, d_coff, max_chunks, cond, cond_on);
    EXH_CUDA_TRY(cudaGetLastError());
    return EXH_OK;
  };
  if (np > SORT_SMALL) {
    k_qs_chunks<<<1, QS_CHUNK_T, 0, st>>>(ctl, d_next, d_segs, d_cfirst, d_cseg, d_coff, max_chunks, 0, 0);
    count_launch(1);
    if (timing_on()) {
      // kernel-class timing: the levels launched one by one, the host checks
      // the counters every few levels; the level loop is one timed unit whose
      // algorithmic bytes are one read and one write of key and id (16 B) per
      // element partitioned
      constexpr int LEVELS_PER_CHECK = 4;
      KTimer kt(KC_SORT, st, 0.0);
      for (int lv = 0;; lv++) {
        EXH_TRY(level(lv & 1, st, 0, 0));
        count_launch(8);
        if ((lv + 1) % LEVELS_PER_CHECK == 0) {
          EXH_CUDA_TRY(cudaMemcpyAsync(&hc, ctl, sizeof(SortCtl), cudaMemcpyDeviceToHost, st));
          EXH_CUDA_TRY(cudaStreamSynchronize(st));
          if (hc.err) break;
          if (hc.nseg == 0 || hc.maxseg <= MID_MAX) {
            kt.bytes = 16.0 * (double)hc.elems;
            break;
          }
        }
        if (lv > np) break;
      }
    } else {
      // the level loop as a graph: a while node over two levels (even and
      // odd buffer) that the last kernel ends on the device; captured once
      // per set of buffers and sizes, launched again only when it stopped at
      // its iteration cap
      std::string key;
      const void* ptrs[16] = {k0, i0, k1, i1, fk, fi, lam, chain, j2, ctl, d_segs, d_next, d_small, d_single, d_cseg,
                              d_cL};
      const int sizes[4] = {max_segs, max_chunks, cap_small, SORT_ITERS_PER_LAUNCH};
      key.append(reinterpret_cast<const char*>(ptrs), sizeof(ptrs));
      key.append(reinterpret_cast<const char*>(sizes), sizeof(sizes));
      if (!c.sort_graph || key != c.sort_graph_key) {
        if (c.sort_graph) cudaGraphExecDestroy(c.sort_graph);
        if (c.sort_graph_src) cudaGraphDestroy(c.sort_graph_src);
        c.sort_graph = nullptr;
        c.sort_graph_src = nullptr;
        c.sort_graph_key.clear();
        EXH_TRY(build_while_graph(
            c,
            [&](cudaStream_t s, cudaGraphConditionalHandle h) -> int {
              EXH_TRY(level(0, s, h, 0));
              return level(1, s, h, 1);
            },
            &c.sort_graph_src, &c.sort_graph));
        c.sort_graph_key = key;
      }
      int done_iters = 0;
      for (int launch = 0;; launch++) {
        EXH_CUDA_TRY(cudaGraphLaunch(c.sort_graph, st));
        EXH_CUDA_TRY(cudaMemcpyAsync(&hc, ctl, sizeof(SortCtl), cudaMemcpyDeviceToHost, st));
        EXH_CUDA_TRY(cudaStreamSynchronize(st));
        count_launch(16 * (hc.iters - done_iters));
        done_iters = hc.iters;
        if (hc.err || hc.nseg == 0 || hc.maxseg <= MID_MAX) break;
        if ((size_t)launch * 2 * SORT_ITERS_PER_LAUNCH > (size_t)np + 4) break;
      }
    }
    if (!hc.err && hc.nseg > 0 && hc.maxseg <= MID_MAX) {
      // the remaining large segments, one block each
      SortBufs mb{{kb[0], kb[1]}, {ib[0], ib[1]}};
      { KTimer kt(KC_SORT, st, 0.0);
      k_qs_mid<<<hc.nseg, MID_T, 0, st>>>(d_segs, ctl, mb, lam, j2, fk, fi, d_small, d_single, cap_small); }
      count_launch(1);
      EXH_CUDA_TRY(cudaGetLastError());
      EXH_CUDA_TRY(cudaMemcpyAsync(&hc, ctl, sizeof(SortCtl), cudaMemcpyDeviceToHost, st));
      EXH_CUDA_TRY(cudaStreamSynchronize(st));
      hc.nseg = 0;
    }
    if (c.verbose) {
      printf("  sort levels done: %d small segments, %d single\n", hc.nsmall, hc.nsingle);
      fflush(stdout);
    }
    if (hc.err) {
      exh_set_error_msg("peak sort: segment lists overflowed", __FILE__, __LINE__);
      return EXH_E_RANGE;
    }
    if (hc.nseg != 0) {
      exh_set_error_msg("peak sort made no progress", __FILE__, __LINE__);
      return EXH_E_TIMEOUT;
    }
  }
  SortBufs sb{{kb[0], kb[1]}, {ib[0], ib[1]}};
  if (hc.nsingle > 0) {
    k_qs_copy_single<<<exh_div_up(hc.nsingle, 256), 256, 0, st>>>(d_single, ctl, sb, fk, fi);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  if (hc.nsmall > 0) {
    const int ns = hc.nsmall;
    const size_t sm = (size_t)SORT_SMALL * (4 * 4 + 2 * 4) + sizeof(int) * 3 * (size_t)SORT_SMALL;
    EXH_CUDA_TRY(set_smem(k_qs_small, sm));
    SmallSortBuffers smb{{kb[0], kb[1]}, {ib[0], ib[1]}};
    { KTimer kt(KC_SORT, st, 16.0 * np);
    k_qs_small<<<ns, SORT_T, sm, st>>>(d_small, ns, smb, fk, fi, &ctl->err); }
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
    int herr = 0;
    EXH_CUDA_TRY(cudaMemcpyAsync(&herr, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr) {
      exh_set_error_msg("peak sort: a block segment did not finish", __FILE__, __LINE__);
      return EXH_E_RANGE;
    }
  }
  h->key = fk;
  h->id = fi;
  return EXH_OK;
}

// ------------------------------------------------------------------ growth
struct GrowArgs {
  const float* delta;
  const float* key;        // sorted peaks (ascending)
  const unsigned* id;
  HaloScalars hs;
  const float* Btab;
  ShellTable t;
};

__device__ __forceinline__ size_t cell_at(int x0, int y0, int z0, int off, const HaloScalars& hs) {
  int i, j, k;
  unpack_off(off, i, j, k);
  return ((size_t)exh_wrap(x0, i, hs.n0) * hs.n1 + exh_wrap(y0, j, hs.n1)) * hs.n2 + exh_wrap(z0, k, hs.n2);
}
__device__ __forceinline__ void peak_coords(unsigned cell, const HaloScalars& hs, int& x, int& y, int& z) {
  z = (int)(cell % hs.n2);
  const unsigned r = cell / hs.n2;
  y = (int)(r % hs.n1);
  x = (int)(r / hs.n1);
}

// Growth + shrink of find_halos.c:274-337 by one warp.  Lanes gather the
// cells of a shell 32 at a time into a per-warp buffer; lane 0 alone adds
// them to the running mean in shell order, so the double arithmetic is the
// reference's sequential loop (and FP64 work is done once, not per lane).
// Integer state is kept identical in all lanes; decisions that depend on the
// mean are broadcast from lane 0.
// Returns 0 ok, 1 count beyond the sigma table, 2 shell beyond the tables;
// gexit is the last shell read (the rejected one).
// Claimed cells during growth, one bit per cell (ng / 32 words, about 2 MB
// at 256^3, resident in L2): set wherever a committing peak writes a flag, and
// flags are only ever added while the halos grow, so a set bit is exactly a
// flag other than FLAG_FREE.  The growth passes test the bit instead of
// reading the 4-byte flag beside every density value.
__device__ __forceinline__ bool cell_claimed(const unsigned* __restrict__ claimed, size_t cell) {
  return (__ldg(&claimed[cell >> 5]) >> (cell & 31)) & 1u;
}
__device__ __forceinline__ void claim_cell(unsigned* claimed, size_t cell) {
  atomicOr(&claimed[cell >> 5], 1u << (cell & 31));
}

__device__ int grow_warp(const GrowArgs& A, const unsigned* __restrict__ claimed, int x0, int y0, int z0, float pden,
                         int lane, double* wbuf, int& count_out, int& gtmp_out, int& gexit_out) {
  const HaloScalars& hs = A.hs;
  double den = (double)pden, den_tmp = (double)pden;     // meaningful in lane 0
  int count = 0, count_tmp = 1, grows_tmp = 0, grows = 0;
  const double bmin = (double)hs.Bmin, mneg = -(double)hs.Mtot;
  while (__shfl_sync(0xffffffffu, (int)(den_tmp >= bmin), 0)) {
    if (count < count_tmp) grows = grows_tmp;
    grows_tmp++;
    den = den_tmp;
    count = count_tmp;
    if (count >= hs.Ncells || grows_tmp > A.t.gmax) {
      count_out = count;
      gtmp_out = grows_tmp;
      gexit_out = A.t.gmax;
      return count >= hs.Ncells ? 1 : 2;
    }
    if (lane == 0) den_tmp = __dmul_rn(den, (double)count);
    const int s0 = A.t.start_cap[grows_tmp], s1 = A.t.start_cap[grows_tmp + 1];
    for (int base = s0; base < s1; base += 32) {
      const int q = base + lane;
      if (q < s1) {
        const size_t cell = cell_at(x0, y0, z0, A.t.off_cap[q], hs);
        wbuf[lane] = cell_claimed(claimed, cell) ? mneg : (double)A.delta[cell];
      }
      __syncwarp();
      const int n = min(32, s1 - base);
      if (lane == 0)
        for (int j = 0; j < n; j++) den_tmp = __dadd_rn(den_tmp, wbuf[j]);
      __syncwarp();
      count_tmp += n;
    }
    if (lane == 0) den_tmp = __ddiv_rn(den_tmp, (double)count_tmp);
  }
  const int gexit = grows_tmp;
  while (count > 0 && __shfl_sync(0xffffffffu, (int)(den < (double)A.Btab[count]), 0)) {
    count_tmp = count;
    if (lane == 0) den = __dmul_rn(den, (double)count);
    const int s0 = A.t.start_cap[grows], s1 = A.t.start_cap[grows + 1];
    for (int base = s0; base < s1; base += 32) {
      const int q = base + lane;
      if (q < s1) wbuf[lane] = (double)A.delta[cell_at(x0, y0, z0, A.t.off_cap[q], hs)];
      __syncwarp();
      const int n = min(32, s1 - base);
      if (lane == 0)
        for (int j = 0; j < n; j++) den = __dsub_rn(den, wbuf[j]);
      __syncwarp();
      count -= n;
    }
    if (lane == 0 && count > 0) den = __ddiv_rn(den, (double)count);
    if (count < count_tmp) grows_tmp = grows;
    grows--;
  }
  count_out = count;
  gtmp_out = grows_tmp;
  gexit_out = gexit;
  return 0;
}

// The same growth and shrink in FP32 with a running bound on the distance
// between the FP32 mean and the reference's FP64 mean.  The outcome (count,
// grows_tmp and the last shell read) depends only on the comparisons with
// the barrier; when every comparison clears the bound, the outcome equals
// the FP64 one and no FP64 arithmetic is needed.  Returns 3 when a
// comparison falls inside the bound (the caller then runs grow_warp).
// A claimed cell in a shell contributes -Mtot, far below any sum of
// densities, so such a shell is rejected with certainty.
struct FBound {
  float f, e;   // value and bound on |f - reference double value|
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) v += __shfl_xor_sync(0xffffffffu, v, w);
  return v;
}

// (prev * c + S) / cn with S a sum of n values (|.| summed to sabs), depth
// the longest chain of float additions that formed S; the reference adds the
// n values one after the other in double
__device__ __forceinline__ FBound fb_update(FBound prev, int c, float S, float sabs, int depth, int n, int cn,
                                            float sign) {
  const float u = 5.9604645e-08f;                  // 2^-24
  const float ud = 1.2e-16f;                       // > 2^-53
  const float fc = (float)c, fcn = (float)cn;
  const float prod = prev.f * fc;
  const float num = prod + sign * S;
  const float res = num / fcn;
  // float side: product, the additions inside S and the final add/divide;
  // double side: the same operations at 2^-53, n additions on partial sums
  // bounded by |prod| + sabs
  const float mag = fabsf(prod) + sabs;
  float e = prev.e * fc + u * fabsf(prod) + (depth + 1) * u * mag + ud * (n + 3) * mag;
  e = e / fcn + 2.f * u * fabsf(res) + ud * fabsf(res);
  return FBound{res, e * 1.01f + 1e-30f};
}

// +1: f >= t for sure, 0: f < t for sure, -1: undecided
__device__ __forceinline__ int fb_ge(FBound b, float t) {
  const float slack = b.e + 3.6e-07f * (fabsf(b.f) + fabsf(t));
  if (b.f - t >= slack) return 1;
  if (t - b.f > slack) return 0;
  return -1;
}

// The same growth with FP64 sums and a bound on the distance to the
// reference's sequential FP64 loop (its sums are formed in another order):
// used where the FP32 bound could not decide, so that the exact sequential
// replay (grow_warp) runs only for a comparison within about 1e-15 of the
// barrier.  Reference and own roundings of the product, the sums (the
// reference's n sequential additions, our depth) and the division, at
// u = 2^-53 (taken as 1.2e-16).
struct DBound {
  double f, e;
};
__device__ __forceinline__ DBound db_update(DBound prev, int c, double S, double sabs, int depth, int n, int cn,
                                            double sign) {
  const double u = 1.2e-16;
  const double fc = (double)c, fcn = (double)cn;
  const double prod = __dmul_rn(prev.f, fc);
  const double res = __ddiv_rn(__dadd_rn(prod, sign * S), fcn);
  const double mag = fabs(prod) + sabs;
  double e = prev.e * fc + 2.0 * u * fabs(prod) + (double)(depth + n + 2) * u * mag;
  e = e / fcn + 2.0 * u * fabs(res);
  return DBound{res, e * 1.01 + 1e-300};
}
__device__ __forceinline__ int db_ge(DBound b, double t) {
  const double slack = b.e + 2.4e-16 * (fabs(b.f) + fabs(t));
  if (b.f - t >= slack) return 1;
  if (t - b.f > slack) return 0;
  return -1;
}

// the two bound tiers behind one interface
template <typename T> struct Tier;
template <> struct Tier<float> {
  using B = FBound;
  static constexpr float U = 5.9604645e-08f;           // 2^-24
  __device__ static B init(float v) { return FBound{v, 0.f}; }
  __device__ static B update(B p, int c, float S, float sa, int depth, int n, int cn, float sign) {
    return fb_update(p, c, S, sa, depth, n, cn, sign);
  }
  __device__ static int ge(B b, float t) { return fb_ge(b, t); }
};
template <> struct Tier<double> {
  using B = DBound;
  static constexpr double U = 1.2e-16;                 // > 2^-53
  __device__ static B init(float v) { return DBound{(double)v, 0.0}; }
  __device__ static B update(B p, int c, double S, double sa, int depth, int n, int cn, double sign) {
    return db_update(p, c, S, sa, depth, n, cn, sign);
  }
  __device__ static int ge(B b, float t) { return db_ge(b, (double)t); }
};

template <typename T> __device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) v += __shfl_xor_sync(0xffffffffu, v, w);
  return v;
}

// Shell sums of the warp growth, kept per warp in shared memory (shell g <
// GW_CACHE at slot g): the growth loads up to GW_CHUNK cells of consecutive
// whole shells in one round trip instead of one round trip per shell, and
// the shrink re-reads nothing.  The sums are of type T (float for the FP32
// tier, double for the FP64 one) in the same storage.
constexpr int GW_U = 4;                  // consecutive cells per lane in a chunk
constexpr int GW_CHUNK = 32 * GW_U;      // cells loaded per round trip
constexpr int GW_CACHE = 256;            // shells a warp keeps
struct ShellCache {
  double sbuf[GW_CACHE], sabuf[GW_CACHE];   // sum and sum of |.| of the shell's densities (T), then their prefixes
  int cnt[GW_CACHE];                        // cells up to and including the shell (prefix of the shell sizes, + 1)
  unsigned short nf[GW_CACHE];              // claimed cells in the shell
  unsigned char depth[GW_CACHE];            // longest chain of additions that formed the sum
  int bnd[32];                              // chunk: first cell of each shell, relative
  template <typename T> __device__ T* s() { return reinterpret_cast<T*>(sbuf); }
  template <typename T> __device__ T* sa() { return reinterpret_cast<T*>(sabuf); }
};

// shell g by lane-strided loads (a shell of more than GW_CHUNK cells, or one
// the cache does not hold)
template <typename T>
__device__ __forceinline__ void shell_direct(const GrowArgs& A, const unsigned* __restrict__ claimed, int x0, int y0,
                                             int z0, int g, int lane, T& s, T& sa, int& nf, int& depth) {
  const int s0 = A.t.start_cap[g], s1 = A.t.start_cap[g + 1];
  T ls = 0, lsa = 0;
  int lf = 0;
#pragma unroll 4
  for (int q = s0 + lane; q < s1; q += 32) {
    const size_t cell = cell_at(x0, y0, z0, A.t.off_cap[q], A.hs);
    lf += cell_claimed(claimed, cell) ? 1 : 0;
    const T v = (T)A.delta[cell];
    ls += v;
    lsa += v < 0 ? -v : v;
  }
  s = warp_sum_t<T>(ls);
  sa = warp_sum_t<T>(lsa);
  nf = __reduce_add_sync(0xffffffffu, lf);
  depth = (s1 - s0 + 31) / 32 + 5;
}

// Shells g0 .. g0 + K - 1 into the cache: as many whole shells as fit in
// GW_CHUNK cells (and below GW_CACHE, at most gmax, K <= 31), loaded in one
// round trip, each lane GW_U consecutive cells; the per-shell sums by a
// segmented scan (within the lane, then across lanes, then the carry into
// the lane's first shell): any term passes through at most
// (GW_U - 1) + 5 + 1 additions.  Returns K (0: shell g0 alone is larger).
template <typename T>
__device__ int shell_chunk(const GrowArgs& A, const unsigned* __restrict__ claimed, int x0, int y0, int z0, int g0,
                           int lane, ShellCache& C) {
  constexpr unsigned FULL = 0xffffffffu;
  T* Cs = C.s<T>();
  T* Csa = C.sa<T>();
  const int base = A.t.start_cap[g0];
  const int gk = g0 + lane;                         // lane k: do shells g0 .. g0 + k fit?
  const bool fit = lane < 31 && gk <= A.t.gmax && gk < GW_CACHE && A.t.start_cap[gk + 1] - base <= GW_CHUNK;
  const int K = __popc(__ballot_sync(FULL, fit));  // the fits are a prefix of the lanes
  if (K == 0) return 0;
  if (lane <= K) C.bnd[lane] = A.t.start_cap[g0 + lane] - base;
  if (lane < K) {                                   // empty shells (r^2 = 7, 15, ...) keep these
    Cs[g0 + lane] = 0;
    Csa[g0 + lane] = 0;
    C.nf[g0 + lane] = 0;
    C.depth[g0 + lane] = 1;
  }
  __syncwarp();
  const int nC = C.bnd[K];
  const int e0 = GW_U * lane;
  int k = 0;
  {
    int hi = K;                                     // last k with bnd[k] <= e0
    while (hi - k > 1) {
      const int mid = (k + hi) >> 1;
      if (C.bnd[mid] <= e0) k = mid; else hi = mid;
    }
  }
  int sh[GW_U];
#pragma unroll
  for (int u = 0; u < GW_U; u++) {
    const int e = e0 + u;
    while (k + 1 < K && C.bnd[k + 1] <= e) k++;
    sh[u] = e < nC ? k : K;                         // past the chunk: a segment of its own
  }
  T v[GW_U];
  int f[GW_U];
#pragma unroll
  for (int u = 0; u < GW_U; u++) {
    v[u] = 0;
    f[u] = 0;
    if (e0 + u < nC) {
      const size_t cell = cell_at(x0, y0, z0, A.t.off_cap[base + e0 + u], A.hs);
      f[u] = cell_claimed(claimed, cell) ? 1 : 0;
      v[u] = (T)A.delta[cell];
    }
  }
  // runs of one shell within the lane
  T rs[GW_U], ra[GW_U];
  int rf[GW_U];
  rs[0] = v[0]; ra[0] = v[0] < 0 ? -v[0] : v[0]; rf[0] = f[0];
#pragma unroll
  for (int u = 1; u < GW_U; u++) {
    const bool same = sh[u] == sh[u - 1];
    const T av = v[u] < 0 ? -v[u] : v[u];
    rs[u] = same ? rs[u - 1] + v[u] : v[u];
    ra[u] = same ? ra[u - 1] + av : av;
    rf[u] = same ? rf[u - 1] + f[u] : f[u];
  }
  // segmented inclusive scan of the lanes' last runs
  const int kF = sh[0], kL = sh[GW_U - 1];
  const int pk = __shfl_up_sync(FULL, kL, 1);
  int hd = (lane == 0 || kF != kL || pk != kF) ? 1 : 0;
  T ts = rs[GW_U - 1], ta = ra[GW_U - 1];
  int tf = rf[GW_U - 1];
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T ys = __shfl_up_sync(FULL, ts, d), ya = __shfl_up_sync(FULL, ta, d);
    const int yf = __shfl_up_sync(FULL, tf, d), yh = __shfl_up_sync(FULL, hd, d);
    if (lane >= d && !hd) {
      ts = ys + ts;
      ta = ya + ta;
      tf = yf + tf;
      hd = yh;
    }
  }
  // carry into the lane's first shell, then the totals at each shell's last cell
  const T cs = __shfl_up_sync(FULL, ts, 1), ca = __shfl_up_sync(FULL, ta, 1);
  const int cf = __shfl_up_sync(FULL, tf, 1);
  const bool carry = lane > 0 && pk == kF;
  const int nk = __shfl_down_sync(FULL, kF, 1);
#pragma unroll
  for (int u = 0; u < GW_U; u++) {
    const bool last = (u + 1 < GW_U) ? sh[u + 1] != sh[u] : (lane == 31 || nk != sh[u]);
    if (last && sh[u] < K) {
      const bool c = carry && sh[u] == kF;
      const int g = g0 + sh[u];
      Cs[g] = c ? cs + rs[u] : rs[u];
      Csa[g] = c ? ca + ra[u] : ra[u];
      C.nf[g] = (unsigned short)(c ? cf + rf[u] : rf[u]);
      C.depth[g] = (unsigned char)(GW_U + 6);
    }
  }
  __syncwarp();
  return K;
}

// Growth and shrink of one peak by a warp with the bound tier T (FP32, or
// FP64 where FP32 could not decide); 3 when a comparison falls inside the
// bound (the next tier then redoes the peak).
//
// The reference's running mean after shells 1..g are accepted is, in exact
// arithmetic, P_g / C_g with P_g = den_peak + (sum of the densities of
// shells 1..g) and C_g = 1 + (cells of shells 1..g), whichever way it was
// reached (grown, or shrunk back from a larger g); its own FP64 recursion
// stays within (C_g + 2 g + 2) 2^-53 (|den_peak| + SA_g) / C_g of that,
// SA_g the prefix of the shells' sums of |density|.  A warp takes up to 31
// consecutive shells at once (lane j: shell g0 + j; a window is the shells
// of one chunk, so nothing past the stopping shell's chunk is loaded), forms
// P_g, SA_g and C_g by warp scans (any term of P_g passes through at most D
// additions: its shell sum's depth, the scan's 5, the FP64 carry from the
// earlier windows and the rounding to T), and compares P_g / C_g with the
// barrier with the bound
// 1.05 (D U_T (|den_peak| + SA_g) / C_g + 2 U_T |den| + the reference's
// share): the first shell where the sequential loop would stop (the size or
// table limit, a claimed cell, a mean below the barrier, or a comparison
// inside the bound) ends the growth.  The shrink then steps down the
// nonempty shells with the stored prefixes.  The outputs are the sequential
// loop's (count, the last removed nonempty shell or gexit, gexit).
// P / C against t with our rounding (D additions at U_T on magnitudes up to
// pabs + SA, and the division) and the reference's (ref_ops FP64 roundings
// on magnitudes up to ref_mag)
template <typename T>
__device__ __forceinline__ int tier_decide(T P, T SA, int Cg, T pabs, int D, int ref_ops, T ref_mag, float t) {
  constexpr T U = Tier<T>::U;
  const T den = P / (T)Cg;
  const T mag = pabs + SA;
  const T e = (T)1.05 * (((T)D * U * mag + (T)ref_ops * (T)1.2e-16 * ref_mag) / (T)Cg +
                         (T)2 * U * (den < 0 ? -den : den)) + (T)1e-30;
  const T tt = (T)t;
  const T slack = e + (T)2 * U * ((den < 0 ? -den : den) + (tt < 0 ? -tt : tt));
  if (den - tt >= slack) return 1;
  if (tt - den > slack) return 0;
  return -1;
}

template <typename T>
__device__ int grow_warp_tier(const GrowArgs& A, const unsigned* __restrict__ claimed, int x0, int y0, int z0,
                              float pden, int lane, ShellCache& C, int& count_out, int& gtmp_out, int& gexit_out) {
  constexpr unsigned FULL = 0xffffffffu;
  const HaloScalars& hs = A.hs;
  T* Ps = C.s<T>();
  T* SAs = C.sa<T>();
  const T p0 = (T)pden, pabs = p0 < 0 ? -p0 : p0;
  // the first test of the loop: the peak's own value against the barrier
  {
    const int d = tier_decide<T>(p0, (T)0, 1, pabs, 1, 2, pabs, hs.Bmin);
    if (d < 0) return 3;
    if (d == 0) { count_out = 0; gtmp_out = 0; gexit_out = 0; return 0; }
  }
  __syncwarp();
  if (lane == 0) { Ps[0] = p0; SAs[0] = (T)0; C.cnt[0] = 1; }
  // prefixes carried from window to window in FP64: each window's sums
  // enter them once, so a term's chain of additions does not grow with the
  // number of windows (depth: its shell sum's, the window scan's 5, the carry
  // and the rounding of P to T)
  double carP = (double)p0, carSA = 0.0;
  int carC = 1, D = 1;
  int gstar = -1, kind = 0;
  for (int gw = 1; gstar < 0;) {
    // the window: the shells of one chunk (at most 128 cells), or one large
    // shell, or past the table the limit alone
    int Kw = 1;
    if (gw <= A.t.gmax) {
      if (gw >= GW_CACHE) return 3;                    // beyond the cache: the next tier
      const int K = shell_chunk<T>(A, claimed, x0, y0, z0, gw, lane, C);
      if (K == 0) {
        T s1, sa1;
        int nf1, d1;
        shell_direct<T>(A, claimed, x0, y0, z0, gw, lane, s1, sa1, nf1, d1);
        if (lane == 0) {
          Ps[gw] = s1; SAs[gw] = sa1;
          C.nf[gw] = (unsigned short)min(nf1, 65535); C.depth[gw] = (unsigned char)min(d1, 255);
        }
        __syncwarp();
      } else {
        Kw = K;
      }
    }
    const int g = gw + lane;
    const bool inwin = lane < Kw;
    const bool exists = inwin && g <= A.t.gmax;
    T S = 0, sa = 0;
    int n = 0, nf = 0, dep = 0;
    if (exists) {
      S = Ps[g]; sa = SAs[g]; nf = C.nf[g]; dep = C.depth[g];
      n = A.t.start_cap[g + 1] - A.t.start_cap[g];
    }
    T pS = S, pA = sa;
    int pn = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T yS = __shfl_up_sync(FULL, pS, o), yA = __shfl_up_sync(FULL, pA, o);
      const int yn = __shfl_up_sync(FULL, pn, o);
      if (lane >= o) { pS += yS; pA += yA; pn += yn; }
    }
    D = max(D, __reduce_max_sync(FULL, dep) + 8);
    const T P = (T)(carP + (double)pS), SA = (T)(carSA + (double)pA);
    const int Cg = carC + pn;
    // events of shell g, in the sequential loop's order: the limits checked
    // when shell g - 1 is accepted, a claimed cell in shell g, then the test
    // of the mean after shell g
    int ev = 0;
    if (inwin) {
      if (!exists) ev = 1;                             // grows_tmp > gmax
      else if (Cg - n >= hs.Ncells) ev = 1;            // count >= Ncells
      else if (nf > 0) ev = 2;
      else {
        const int d = tier_decide<T>(P, SA, Cg, pabs, D, Cg + 2 * g + 2, pabs + SA, hs.Bmin);
        ev = d == 0 ? 3 : (d < 0 ? 4 : 0);
      }
    }
    if (exists) { Ps[g] = P; SAs[g] = SA; C.cnt[g] = Cg; }
    const unsigned evm = __ballot_sync(FULL, ev != 0);
    if (evm) {
      const int l = __ffs(evm) - 1;
      gstar = gw + l;
      kind = __shfl_sync(FULL, ev, l);
    } else {
      carP += (double)__shfl_sync(FULL, pS, Kw - 1);
      carSA += (double)__shfl_sync(FULL, pA, Kw - 1);
      carC += __shfl_sync(FULL, pn, Kw - 1);
    }
    __syncwarp();
    gw += Kw;
  }
  if (kind == 4) return 3;
  // accepted shells 1 .. gstar - 1
  const int count_acc = C.cnt[gstar - 1];
  if (kind == 1) {
    count_out = count_acc;
    gtmp_out = gstar;
    gexit_out = A.t.gmax;
    return count_acc >= hs.Ncells ? 1 : 2;
  }
  const int gexit = gstar;
  // grows: the last accepted shell with cells (0: the peak cell)
  int k = gstar - 1;
  while (k > 0 && C.cnt[k] == C.cnt[k - 1]) k--;
  int count = count_acc, gtmp = gexit;
  // the reference reaches shell k of the shrink by subtracting from the
  // accepted total: its roundings on the accepted magnitude
  const int ref_ops = 2 * count_acc + 4 * gstar + 4;
  const T ref_mag = pabs + SAs[gstar - 1];
  while (count > 0) {
    const int d = tier_decide<T>(Ps[k], SAs[k], C.cnt[k], pabs, D, ref_ops, ref_mag, A.Btab[count]);   // shrink while den < B
    if (d < 0) return 3;
    if (d == 1) break;
    gtmp = k;                                          // shell k removed
    if (k == 0) { count = 0; break; }
    int j = k - 1;
    while (j > 0 && C.cnt[j] == C.cnt[j - 1]) j--;    // the next shell down with cells
    k = j;
    count = C.cnt[k];
  }
  count_out = count;
  gtmp_out = gtmp;
  gexit_out = gexit;
  return 0;
}

constexpr int GROW_T = 256;   // 8 peaks (one per warp) per block
constexpr int LANE_GMAX = 6;          // shells one thread grows through (81 cells) before a warp takes over
constexpr int LANE_COMMIT_MAX = 128;  // reserved cells one thread checks and labels
// Most peaks read shell 1 only (a one-cell halo) and check 7 cells at the
// commit; a warp whose lanes mix them with larger peaks runs as long as its
// largest, so the first thread passes stop there and hand the others to a
// second thread pass, whose warps then hold peaks of similar size.
constexpr int FIRST_GMAX = 1;         // shells the first growth pass grows through
constexpr int FIRST_COMMIT_MAX = 7;   // cells the first commit pass checks (r^2 <= 1)
// The second passes run one thread per peak while many peaks are handed on
// (throughput); with at most MID_WARP_MAX (growth) or COMMIT_WARP_MAX
// (commit) the warp passes take them instead, one warp per peak (a round's
// time is then the longest peak's chain of dependent loads, shorter across a
// warp).  Thresholds from launch timings of the box_256 workload.
constexpr int MID_WARP_MAX = 16384;
constexpr int COMMIT_WARP_MAX = 8192;
constexpr int GROW_PERSIST = EXH_NUM_SMS * 8;   // blocks of the persistent warp passes

__device__ __forceinline__ unsigned resv_key(int tag, int r) { return ((unsigned)tag << 24) | (0xFFFFFFu - (unsigned)r); }

// Appends staged per warp in shared memory: list space is taken 32 entries
// at a time, one atomic per 32 peaks instead of one per warp and step (the
// passes of a round hand on a share of nearly every warp's peaks, and the
// list counters are single words).  Every lane of the warp calls these.
struct WarpStage {
  int v[64];
  int n;
};
__device__ __forceinline__ void stage_push(WarpStage& s, int* list, int* cnt, bool flag, int val, int lane) {
  const unsigned m = __ballot_sync(0xffffffffu, flag);
  if (!m) return;
  const int base = s.n;
  if (flag) s.v[base + __popc(m & ((1u << lane) - 1u))] = val;
  const int nn = base + __popc(m);
  __syncwarp();
  if (nn >= 32) {
    int g = 0;
    if (lane == 0) g = atomicAdd(cnt, 32);
    g = __shfl_sync(0xffffffffu, g, 0);
    list[g + lane] = s.v[lane];
    const int rem = nn - 32;
    const int keep = lane < rem ? s.v[32 + lane] : 0;
    __syncwarp();
    if (lane < rem) s.v[lane] = keep;
    if (lane == 0) s.n = rem;
  } else if (lane == 0) {
    s.n = nn;
  }
  __syncwarp();
}
__device__ __forceinline__ void stage_flush(WarpStage& s, int* list, int* cnt, int lane) {
  const int nn = s.n;
  if (nn > 0) {
    int g = 0;
    if (lane == 0) g = atomicAdd(cnt, nn);
    g = __shfl_sync(0xffffffffu, g, 0);
    if (lane < nn) list[g + lane] = s.v[lane];
  }
  __syncwarp();
  if (lane == 0) s.n = 0;
  __syncwarp();
}

// grow_warp_tier<float> by one thread for the small spheres that most peaks grow:
// the shell sums are sequential (bound depth = cells in the shell).  Returns
// 3 when a comparison is undecided or the growth would pass shell gmax_lane;
// a later pass then redoes the peak from the start.
__device__ int grow_lane_f32(const GrowArgs& A, const unsigned* __restrict__ claimed, int x0, int y0, int z0, float pden,
                             int gmax_lane, int& count_out, int& gtmp_out, int& gexit_out) {
  const HaloScalars& hs = A.hs;
  FBound den{pden, 0.f}, den_tmp{pden, 0.f};
  bool rejected = false;
  int count = 0, count_tmp = 1, grows_tmp = 0, grows = 0;
  while (true) {
    int d = rejected ? 0 : fb_ge(den_tmp, hs.Bmin);
    if (d < 0) return 3;
    if (!d) break;
    if (count < count_tmp) grows = grows_tmp;
    grows_tmp++;
    den = den_tmp;
    count = count_tmp;
    if (count >= hs.Ncells || grows_tmp > A.t.gmax) {
      count_out = count;
      gtmp_out = grows_tmp;
      gexit_out = A.t.gmax;
      return count >= hs.Ncells ? 1 : 2;
    }
    if (grows_tmp > gmax_lane) return 3;
    const int s0 = A.t.start_cap[grows_tmp], s1 = A.t.start_cap[grows_tmp + 1];
    float sm = 0.f, sa = 0.f;
    bool foreign = false;
#pragma unroll 8
    for (int q = s0; q < s1; q++) {
      const size_t cell = cell_at(x0, y0, z0, A.t.off_cap[q], hs);
      foreign |= cell_claimed(claimed, cell);
      const float v = A.delta[cell];
      sm += v;
      sa += fabsf(v);
    }
    const int n = s1 - s0;
    count_tmp += n;
    if (foreign) { rejected = true; continue; }
    den_tmp = fb_update(den, count, sm, sa, n + 5, n, count_tmp, 1.f);
  }
  const int gexit = grows_tmp;
  while (count > 0) {
    const int d = fb_ge(den, A.Btab[count]);
    if (d < 0) return 3;
    if (d == 1) break;
    count_tmp = count;
    const int s0 = A.t.start_cap[grows], s1 = A.t.start_cap[grows + 1];
    float sm = 0.f, sa = 0.f;
#pragma unroll 8
    for (int q = s0; q < s1; q++) {
      const float v = A.delta[cell_at(x0, y0, z0, A.t.off_cap[q], hs)];
      sm += v;
      sa += fabsf(v);
    }
    const int n = s1 - s0;
    count -= n;
    if (count > 0) den = fb_update(den, count_tmp, sm, sa, n + 5, n, count, -1.f);
    if (count < count_tmp) grows_tmp = grows;
    grows--;
  }
  count_out = count;
  gtmp_out = grows_tmp;
  gexit_out = gexit;
  return 0;
}

struct RoundArgs {
  unsigned char* state;
  int* flag;
  unsigned* resv;
  unsigned* claimed;   // one bit per cell: flag != FLAG_FREE
  // device words: the round's reservation tag and the number of peaks (so
  // that the arguments, and a captured round loop, do not change with them)
  const int* tag;
  const long long* np;
  int* cnt;
  int* gtmp;
  int* gexit;
  int* gst;
  int* gfin;
  int* err;
  int* next;        // peaks left for the next round
  int* nnext;
  int* mlist;       // peaks handed from the first growth pass to the second
  int* nm;
  int* wlist;       // peaks handed to the warp growth pass
  int* nw;
  int* c2list;      // peaks handed from the first commit pass to the second
  int* nc2;
  int* clist;       // peaks handed to the warp commit pass
  int* nc;
  int* nexact;      // growths the FP32 bound could not decide (run in FP64)
  unsigned* nwords; // 4-byte words touched per peak (timing only) or null
};

// Reservation of the cells off_all[q0, q1) (step dq) around (x, y, z) with
// key: the current values are read in batches of RB before any atomic, so a
// thread has RB loads in flight instead of one.  Values only grow during a
// round (atomicMax), so a value read early that is already >= key stays so
// and the skipped atomic would not have changed it.
constexpr int RB = 8;
__device__ __forceinline__ void reserve_cells(const GrowArgs& A, unsigned* resv, int x, int y, int z, int q0, int q1,
                                              int dq, unsigned key) {
  for (int qb = q0; qb < q1; qb += RB * dq) {
    size_t cells[RB];
    unsigned v[RB];
#pragma unroll
    for (int u = 0; u < RB; u++) {
      const int q = qb + u * dq;
      cells[u] = q < q1 ? cell_at(x, y, z, A.t.off_all[q], A.hs) : 0;
    }
#pragma unroll
    for (int u = 0; u < RB; u++) v[u] = qb + u * dq < q1 ? resv[cells[u]] : 0xffffffffu;
#pragma unroll
    for (int u = 0; u < RB; u++)
      if (v[u] < key) atomicMax(&resv[cells[u]], key);
  }
}

// true when no cell off_all[q0, q1) (step dq) holds a reservation above key;
// RB loads in flight per batch, the test after each batch
__device__ __forceinline__ bool cells_mine(const GrowArgs& A, const unsigned* resv, int x, int y, int z, int q0, int q1,
                                           int dq, unsigned key) {
  for (int qb = q0; qb < q1; qb += RB * dq) {
    unsigned v[RB];
#pragma unroll
    for (int u = 0; u < RB; u++) {
      const int q = qb + u * dq;
      v[u] = q < q1 ? resv[cell_at(x, y, z, A.t.off_all[q], A.hs)] : 0u;
    }
    bool ok = true;
#pragma unroll
    for (int u = 0; u < RB; u++) ok &= v[u] <= key;
    if (!ok) return false;
  }
  return true;
}

__device__ __forceinline__ unsigned tentative_words(const GrowArgs& A, int ge) {
  // cells read by the growth (density + label) and reserved (read + atomic)
  return 2u * (A.t.start_cap[min(ge, A.t.gmax) + 1] - A.t.start_cap[1]) + 2u * A.t.start_all[ge] + 2u;
}

// One round, part 1 (one thread per pending peak): every pending peak grows
// with the flags committed so far and keeps the result.  Flags are only ever
// added, and a claimed cell can only stop a growth earlier, so the last shell
// read (gexit) is an upper bound of the final one, and the cells the peak
// will flag (r^2 < final grows_tmp <= final gexit) lie inside r^2 < gexit:
// the peak reserves those cells, its possible writes.  FIRST: the round's
// list, growth through shell FIRST_GMAX, larger peaks to the second pass;
// second pass: through shell LANE_GMAX, larger peaks (or a comparison too
// close to call in FP32) to the warp pass.
template <bool FIRST>
__global__ void __launch_bounds__(GROW_T)
k_tentative(GrowArgs A, const int* __restrict__ list, const int* __restrict__ nlist, RoundArgs R) {
  __shared__ WarpStage stg[GROW_T / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = FIRST ? *nlist : *R.nm;
  const int* lst = FIRST ? list : R.mlist;
  int* out = FIRST ? R.mlist : R.wlist;
  int* nout = FIRST ? R.nm : R.nw;
  if (!FIRST && n <= MID_WARP_MAX) return;   // the warp pass takes them
  if (lane == 0) stg[warp].n = 0;
  __syncwarp();
  const int stride = (int)(gridDim.x * blockDim.x);
  for (int base = (int)(blockIdx.x * (size_t)blockDim.x) + warp * 32; base < n; base += stride) {   // warp-uniform
    const int t = base + lane;
    const int r = t < n ? lst[t] : -1;       // first round: -1 also marks a peak below the barrier
    bool hand_on = false;
    if (r >= 0) {
      const int64_t l = *R.np - 1 - r;
      const unsigned cell0 = A.id[l];
      if (FIRST && cell_claimed(R.claimed, cell0)) {   // find_halos.c:233: the peak is already inside a halo
        R.state[r] = 1;
        R.cnt[r] = 0;
      } else {
        int x, y, z;
        peak_coords(cell0, A.hs, x, y, z);
        int count, gt, ge;
        const int st = grow_lane_f32(A, R.claimed, x, y, z, A.key[l], FIRST ? FIRST_GMAX : LANE_GMAX, count, gt, ge);
        if (st == 3) {
          hand_on = true;
        } else {
          R.cnt[r] = count; R.gtmp[r] = gt; R.gexit[r] = ge; R.gst[r] = st;
          if (R.nwords) R.nwords[r] += tentative_words(A, ge);
          const unsigned key = resv_key(*R.tag, r);
          reserve_cells(A, R.resv, x, y, z, 0, A.t.start_all[ge], 1, key);   // cells it may flag: r^2 < gexit
        }
      }
    }
    stage_push(stg[warp], out, nout, hand_on, r, lane);
  }
  stage_flush(stg[warp], out, nout, lane);
}

// part 1, warp pass over the peaks the thread pass handed on (persistent)
__global__ void __launch_bounds__(GROW_T)
k_tentative_warp(GrowArgs A, RoundArgs R) {
  __shared__ double wb[GROW_T / 32][32];
  __shared__ ShellCache cache[GROW_T / 32];
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  // the first pass's hand-offs when few (the thread pass skipped them), then
  // the thread pass's
  const int nmid = *R.nm <= MID_WARP_MAX ? *R.nm : 0;
  const int n = nmid + *R.nw;
  for (int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); w < n; w += nwarps) {
    const int r = w < nmid ? R.mlist[w] : R.wlist[w - nmid];
    const int64_t l = *R.np - 1 - r;
    const unsigned cell0 = A.id[l];
    int x, y, z;
    peak_coords(cell0, A.hs, x, y, z);
    int count, gt, ge;
    ShellCache& C = cache[threadIdx.x >> 5];
    int st = grow_warp_tier<float>(A, R.claimed, x, y, z, A.key[l], lane, C, count, gt, ge);
    if (st == 3) st = grow_warp_tier<double>(A, R.claimed, x, y, z, A.key[l], lane, C, count, gt, ge);
    if (st == 3) {
      if (lane == 0) atomicAdd(R.nexact, 1);
      st = grow_warp(A, R.claimed, x, y, z, A.key[l], lane, wb[threadIdx.x >> 5], count, gt, ge);
    }
    if (lane == 0) { R.cnt[r] = count; R.gtmp[r] = gt; R.gexit[r] = ge; R.gst[r] = st; }
    if (lane == 0 && R.nwords) R.nwords[r] += tentative_words(A, ge);
    const unsigned key = resv_key(*R.tag, r);
    reserve_cells(A, R.resv, x, y, z, lane, A.t.start_all[ge], 32, key);
  }
}

// the commit of a peak that holds every cell it read: the tentative result
// stands (no pending peak of higher rank can change those cells)
__device__ __forceinline__ bool commit_status(const RoundArgs& R, int r) {
  const int st = R.gst[r];
  if (st) {
    atomicMax(R.err, st);
    R.state[r] = 1;
    return false;
  }
  R.state[r] = 1;
  R.gfin[r] = R.gtmp[r];
  return R.cnt[r] != 0;                  // find_halos.c:339-340
}

// One round, part 2: a peak commits when no pending peak of higher rank
// reserved (may flag) any cell it read (r^2 <= gexit): its tentative result
// is then the sequential one.  Reservation keys order by round, then rank,
// so a key above the peak's own is a higher-rank writer of this round.
// FIRST: the round's list, peaks that read at most FIRST_COMMIT_MAX cells,
// the others to the second pass; second pass: at most LANE_COMMIT_MAX cells,
// the others to the warp pass.
template <bool FIRST>
__global__ void __launch_bounds__(GROW_T)
k_commit(GrowArgs A, const int* __restrict__ list, const int* __restrict__ nlist, RoundArgs R) {
  __shared__ WarpStage stg_on[GROW_T / 32], stg_next[GROW_T / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = FIRST ? *nlist : *R.nc2;
  const int* lst = FIRST ? list : R.c2list;
  int* out = FIRST ? R.c2list : R.clist;
  int* nout = FIRST ? R.nc2 : R.nc;
  if (!FIRST && n <= COMMIT_WARP_MAX) return;   // the warp pass takes them
  if (lane == 0) { stg_on[warp].n = 0; stg_next[warp].n = 0; }
  __syncwarp();
  const int stride = (int)(gridDim.x * blockDim.x);
  for (int base = (int)(blockIdx.x * (size_t)blockDim.x) + warp * 32; base < n; base += stride) {   // warp-uniform
    const int t = base + lane;
    int r = t < n ? lst[t] : -1;
    if (r >= 0 && FIRST && R.state[r]) r = -1;     // resolved by the centre test this round
    bool hand_on = false, retry = false;
    if (r >= 0) {
      const int e = A.t.start_all[R.gexit[r] + 1];
      if (e > (FIRST ? FIRST_COMMIT_MAX : LANE_COMMIT_MAX)) {
        hand_on = true;
      } else {
        const unsigned cell0 = A.id[*R.np - 1 - r];
        int x, y, z;
        peak_coords(cell0, A.hs, x, y, z);
        const unsigned key = resv_key(*R.tag, r);
        const bool mine = cells_mine(A, R.resv, x, y, z, 0, e, 1, key);
        if (R.nwords) R.nwords[r] += (unsigned)e;
        if (!mine) {
          retry = true;
        } else if (commit_status(R, r)) {
          const int we = A.t.start_all[R.gtmp[r]];     // cells with r^2 < grows_tmp
          for (int q = 0; q < we; q++) {
            const size_t cq = cell_at(x, y, z, A.t.off_all[q], A.hs);
            R.flag[cq] = r;
            claim_cell(R.claimed, cq);
          }
          if (R.nwords) R.nwords[r] += (unsigned)we;
          R.flag[cell0] = -(r + 2);
          claim_cell(R.claimed, cell0);
        }
      }
    }
    stage_push(stg_on[warp], out, nout, hand_on, r, lane);
    stage_push(stg_next[warp], R.next, R.nnext, retry, r, lane);
  }
  stage_flush(stg_on[warp], out, nout, lane);
  stage_flush(stg_next[warp], R.next, R.nnext, lane);
}

// part 2, warp pass (persistent) over the peaks handed on by k_commit
__global__ void __launch_bounds__(GROW_T)
k_commit_warp(GrowArgs A, RoundArgs R) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  const int nmid = *R.nc2 <= COMMIT_WARP_MAX ? *R.nc2 : 0;
  const int n = nmid + *R.nc;
  for (int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); w < n; w += nwarps) {
    const int r = w < nmid ? R.c2list[w] : R.clist[w - nmid];
    const unsigned cell0 = A.id[*R.np - 1 - r];
    int x, y, z;
    peak_coords(cell0, A.hs, x, y, z);
    const unsigned key = resv_key(*R.tag, r);
    const int e = A.t.start_all[R.gexit[r] + 1];
    bool mine = true;
    for (int qb = 0; qb < e && mine; qb += 32 * RB)          // warp-uniform: all lanes leave together
      mine = __all_sync(0xffffffffu, cells_mine(A, R.resv, x, y, z, qb + lane, min(qb + 32 * RB, e), 32, key));
    if (lane == 0 && R.nwords) R.nwords[r] += (unsigned)e;
    if (!mine) {
      if (lane == 0) R.next[atomicAdd(R.nnext, 1)] = r;
      continue;
    }
    bool keep = false;
    if (lane == 0) keep = commit_status(R, r);
    if (!__shfl_sync(0xffffffffu, (int)keep, 0)) continue;
    const int we = A.t.start_all[R.gtmp[r]];
    for (int q = lane; q < we; q += 32) {
      const size_t cq = cell_at(x, y, z, A.t.off_all[q], A.hs);
      R.flag[cq] = r;
      claim_cell(R.claimed, cq);
    }
    if (lane == 0 && R.nwords) R.nwords[r] += (unsigned)we;
    __syncwarp();
    if (lane == 0) {
      R.flag[cell0] = -(r + 2);
      claim_cell(R.claimed, cell0);
    }
  }
}

// round bookkeeping on the device: counters of the growth loop in B_HOSTIO2
// ([0] unused, [1] error, [2] [3] the two list lengths, [4] warp growth list,
// [5] warp commit list, [6..7] byte total, [10] second growth list, [11]
// second commit list, [12] FP64 growths, [16] tag, [18..19] peak count)
constexpr int GROW_TAG = 16, GROW_NP = 18, GROW_NM = 10, GROW_NC2 = 11, GROW_NEXACT = 12;
constexpr int GROW_ROUNDS_PER_LAUNCH = 250;     // reservation tags 1..250 (8 bits of the key)

// start of a round with current list `cur`: its next list and the warp
// lists empty, the next reservation tag
__global__ void k_round_begin(int* dcnt, int cur) {
  if (threadIdx.x == 0) {
    dcnt[3 - cur] = 0;
    dcnt[4] = 0;
    dcnt[5] = 0;
    dcnt[GROW_NM] = 0;
    dcnt[GROW_NC2] = 0;
    dcnt[GROW_TAG] += 1;
  }
}

// end of the round loop's body (current list 1): go on while peaks are left,
// no growth failed and the tags last
__global__ void k_round_end(const int* dcnt, cudaGraphConditionalHandle cond) {
  if (threadIdx.x == 0)
    cudaGraphSetConditional(cond, (dcnt[2] > 0 && dcnt[1] == 0 && dcnt[GROW_TAG] < GROW_ROUNDS_PER_LAUNCH - 1) ? 1u
                                                                                                               : 0u);
}

__global__ void k_sum_words(const unsigned* __restrict__ w, int n, unsigned long long* __restrict__ out) {
  unsigned long long s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += w[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// The first round's list in cell order: the processed peak of rank r
// (sorted index np - 1 - r >= L0) at its position among the peaks in cell
// order (group offset + the mask bits before it), -1 at the others.  Which
// peak a thread grows does not change any result (reservations decide by
// rank); in cell order the threads of a warp grow neighbouring peaks, so
// their shells share sectors in L1 and L2.
__global__ void k_spatial_list(const unsigned* __restrict__ id, long long np, long long L0,
                               const unsigned* __restrict__ mask, const unsigned* __restrict__ off,
                               int* __restrict__ list) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long l = L0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; l < np; l += stride) {
    const unsigned cell = id[l];
    const unsigned w = cell >> 5;
    unsigned p = off[cell / PK_T];
    for (unsigned q = (cell / PK_T) * (PK_T / 32); q < w; q++) p += __popc(__ldg(&mask[q]));
    p += __popc(__ldg(&mask[w]) & ((1u << (cell & 31)) - 1u));
    list[p] = (int)(np - 1 - l);
  }
}

__global__ void k_kept(const int* __restrict__ cnt, const unsigned char* __restrict__ state, int nproc, int Nmin,
                       int* __restrict__ kept) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nproc) return;
  kept[r] = (cnt[r] > 0 && cnt[r] >= Nmin) ? 1 : 0;
}

__global__ void k_halo_index(const int* __restrict__ kept, const int* __restrict__ hid_ex, int nproc,
                             int* __restrict__ hid, int* __restrict__ hpeak) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nproc) return;
  if (kept[r]) {
    hid[r] = hid_ex[r];
    hpeak[hid_ex[r]] = r;
  } else {
    hid[r] = -1;
  }
}

__global__ void k_lower_bound(const float* __restrict__ key, int64_t n, float v, long long* out) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) / 2;
    if (key[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  *out = lo;
}

int grow_halos(Ctx& c, const float* delta, const BoxParams& b, const HaloScalars& hs, const float* Btab_dev,
               const ShellTable& t, HaloDev* h, cudaStream_t st) {
  const int64_t np = h->np;
  // the reference loop visits sorted indices np-1 .. 1 while den >= Bmin
  int64_t nproc = 0;
  if (np >= 2) {
    // lower bound of Bmin in the ascending keys
    EXH_TRY(c.buf[B_HOSTIO2].ensure(64));
    long long* dlb = c.buf[B_HOSTIO2].as<long long>();
    k_lower_bound<<<1, 1, 0, st>>>(h->key, np, hs.Bmin, dlb);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
    long long lo = 0;
    EXH_CUDA_TRY(cudaMemcpyAsync(&lo, dlb, sizeof(lo), cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    const int64_t L0 = std::max<int64_t>(lo, 1);
    nproc = np - L0;
  }
  h->nproc = nproc;
  if (nproc >= (1 << 24) - 1) {
    exh_set_error_msg("more than 2^24 peaks above the barrier", __FILE__, __LINE__);
    return EXH_E_UNSUPPORTED;
  }
  const size_t ng = b.ng;
  const size_t npr = std::max<int64_t>(nproc, 1);
  const size_t nclaim = ng / 32 + 1;
  EXH_TRY(c.buf[B_FLAG].ensure(sizeof(int) * ng * 2 + sizeof(unsigned) * nclaim));
  h->flag = c.buf[B_FLAG].as<int>();
  h->resv = reinterpret_cast<unsigned*>(h->flag + ng);
  unsigned* claimed = h->resv + ng;
  // per processed peak arrays, laid out by the buffer's capacity (stable
  // addresses from one realisation to the next)
  EXH_TRY(c.buf[B_HALO].ensure(npr * (sizeof(int) * 8 + 1) + 64));
  const size_t hcap = (c.buf[B_HALO].cap - 64) / (sizeof(int) * 8 + 1);
  h->gfree = c.buf[B_HALO].as<int>();
  h->gfin = h->gfree + hcap;
  h->cnt = h->gfin + hcap;
  h->hid = h->cnt + hcap;
  h->hpeak = h->hid + hcap;
  int* kept = h->hpeak + hcap;
  int* misc = kept + hcap;            // hcap ints: scan scratch / counters
  h->words = reinterpret_cast<unsigned*>(misc + hcap);
  h->state = reinterpret_cast<unsigned char*>(h->words + hcap);
  EXH_CUDA_TRY(cudaMemsetAsync(h->flag, 0xff, sizeof(int) * ng, st));      // FLAG_FREE
  EXH_CUDA_TRY(cudaMemsetAsync(h->resv, 0, sizeof(unsigned) * ng, st));
  EXH_CUDA_TRY(cudaMemsetAsync(claimed, 0, sizeof(unsigned) * nclaim, st));
  EXH_CUDA_TRY(cudaMemsetAsync(h->state, 0, npr, st));
  EXH_CUDA_TRY(cudaMemsetAsync(h->cnt, 0, sizeof(int) * npr, st));
  h->nh = 0;
  if (nproc == 0) return EXH_OK;
  GrowArgs A{delta, h->key, h->id, hs, Btab_dev, t};
  const unsigned nb = exh_div_up(nproc, 128);
  if (c.verbose) { printf("  %lld peaks above the barrier\n", (long long)nproc); fflush(stdout); }
  // per processed peak during the rounds: gfree = last shell read,
  // kept = growth status; both are rewritten after the rounds
  int* gexit = h->gfree;
  int* gst = kept;
  EXH_TRY(c.buf[B_HOSTIO2].ensure(128));
  int* dcnt = c.buf[B_HOSTIO2].as<int>();
  // pending peaks as lists: the first round's in cell order with gaps
  // (np entries), then compacted lists (hid serves as the second list during
  // the rounds and is rewritten afterwards); the hand-off lists of the later
  // passes and the first list live in the hand-off buffer, in fifths of its
  // capacity
  const size_t lcap = std::max<size_t>(npr, (size_t)np);
  EXH_TRY(c.buf[B_HALO3].ensure(sizeof(int) * 5 * lcap));
  const size_t fifth = c.buf[B_HALO3].cap / (5 * sizeof(int));
  int* wlist = c.buf[B_HALO3].as<int>();
  int* clist = wlist + fifth;
  int* mlist = clist + fifth;
  int* c2list = mlist + fifth;
  int* lists[2] = {c2list + fifth, h->hid};
  {
    unsigned *pmask, *pcnt, *poff;
    peak_mask_layout(c, ng, &pmask, &pcnt, &poff);
    EXH_CUDA_TRY(cudaMemsetAsync(lists[0], 0xff, sizeof(int) * (size_t)np, st));
    k_spatial_list<<<exh_div_up(nproc, 256), 256, 0, st>>>(h->id, np, np - nproc, pmask, poff, lists[0]);
    count_launch(1);
    EXH_CUDA_TRY(cudaGetLastError());
  }
  {
    int init[20] = {0, 0, (int)np, 0, 0, 0};
    const long long npl = np;
    std::memcpy(&init[GROW_NP], &npl, sizeof(npl));
    EXH_TRY(upload_small(dcnt, init, sizeof(init), st));
  }
  if (timing_on()) EXH_CUDA_TRY(cudaMemsetAsync(h->words, 0, sizeof(unsigned) * npr, st));
  KTimer kt(KC_GROW, st, 0.0);   // the whole growth phase is one timed unit
  // persistent grids, sized by the peak buffers' capacity (stable from one
  // realisation to the next)
  const unsigned nbl = std::min<unsigned>(exh_div_up(std::max<size_t>(peak_cap(c), 1), GROW_T), GROW_PERSIST);
  auto round = [&](int cur, cudaStream_t s) -> int {
    RoundArgs R;
    R.state = h->state; R.flag = h->flag; R.resv = h->resv; R.claimed = claimed;
    R.tag = dcnt + GROW_TAG;
    R.np = reinterpret_cast<const long long*>(dcnt + GROW_NP);
    R.cnt = h->cnt; R.gtmp = h->gfin; R.gexit = gexit; R.gst = gst; R.gfin = h->gfin;
    R.err = dcnt + 1; R.next = lists[cur ^ 1]; R.nnext = dcnt + 3 - cur;
    R.wlist = wlist; R.nw = dcnt + 4; R.clist = clist; R.nc = dcnt + 5;
    R.mlist = mlist; R.nm = dcnt + GROW_NM; R.c2list = c2list; R.nc2 = dcnt + GROW_NC2;
    R.nexact = dcnt + GROW_NEXACT;
    R.nwords = timing_on() ? h->words : nullptr;
    const int* ncur = dcnt + 2 + cur;
    k_round_begin<<<1, 32, 0, s>>>(dcnt, cur);
    k_tentative<true><<<nbl, GROW_T, 0, s>>>(A, lists[cur], ncur, R);
    k_tentative<false><<<nbl, GROW_T, 0, s>>>(A, lists[cur], ncur, R);
    k_tentative_warp<<<nbl, GROW_T, 0, s>>>(A, R);
    k_commit<true><<<nbl, GROW_T, 0, s>>>(A, lists[cur], ncur, R);
    k_commit<false><<<nbl, GROW_T, 0, s>>>(A, lists[cur], ncur, R);
    k_commit_warp<<<nbl, GROW_T, 0, s>>>(A, R);
    EXH_CUDA_TRY(cudaGetLastError());
    return EXH_OK;
  };
  int hc[16] = {};
  if (timing_on()) {
    // kernel-class timing: rounds launched one by one, the host checks every
    // few rounds
    constexpr int ROUNDS_PER_CHECK = 3;
    int cur = 0;
    for (int rd = 0;; rd++) {
      if (rd > 0 && rd % GROW_ROUNDS_PER_LAUNCH == 0) {
        EXH_CUDA_TRY(cudaMemsetAsync(h->resv, 0, sizeof(unsigned) * ng, st));
        EXH_CUDA_TRY(cudaMemsetAsync(dcnt + GROW_TAG, 0, sizeof(int), st));
      }
      EXH_TRY(round(cur, st));
      count_launch(7);
      cur ^= 1;
      if ((rd + 1) % ROUNDS_PER_CHECK == 0) {
        EXH_CUDA_TRY(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
        EXH_CUDA_TRY(cudaStreamSynchronize(st));
        if (c.verbose > 1) { printf("  growth round %d: %d left\n", rd, hc[2 + cur]); fflush(stdout); }
        if (hc[1] || hc[2 + cur] == 0) break;
      }
      if (rd > nproc + 2) {
        exh_set_error_msg("halo growth made no progress", __FILE__, __LINE__);
        return EXH_E_TIMEOUT;
      }
    }
  } else {
    // the round loop as a graph: a while node over two rounds (list 0, then
    // list 1) that k_round_end ends on the device; one graph per set of
    // arguments, a few kept (batches alternate box sizes), launched again
    // with fresh reservation tags only if it stopped at its round cap
    std::string key;
    const void* ptrs[16] = {delta, h->key, h->id, Btab_dev, h->state, h->flag, h->resv, claimed, h->cnt, h->gfin,
                            gexit, gst, dcnt, lists[0], lists[1], wlist};
    key.append(reinterpret_cast<const char*>(ptrs), sizeof(ptrs));
    key.append(reinterpret_cast<const char*>(&clist), sizeof(clist));
    key.append(reinterpret_cast<const char*>(&hs), sizeof(hs));
    key.append(reinterpret_cast<const char*>(&t), sizeof(t));
    key.append(reinterpret_cast<const char*>(&nbl), sizeof(nbl));
    cudaGraphExec_t ex = nullptr;
    for (auto& e : c.grow_graphs)
      if (e.key == key) ex = e.exec;
    if (!ex) {
      if (c.grow_graphs.size() >= 6) {
        cudaGraphExecDestroy(c.grow_graphs.front().exec);
        cudaGraphDestroy(c.grow_graphs.front().src);
        c.grow_graphs.erase(c.grow_graphs.begin());
      }
      Ctx::GraphEntry e;
      EXH_TRY(build_while_graph(
          c,
          [&](cudaStream_t s, cudaGraphConditionalHandle cond) -> int {
            EXH_TRY(round(0, s));
            EXH_TRY(round(1, s));
            k_round_end<<<1, 32, 0, s>>>(dcnt, cond);
            EXH_CUDA_TRY(cudaGetLastError());
            return EXH_OK;
          },
          &e.src, &e.exec));
      e.key = key;
      c.grow_graphs.push_back(e);
      ex = e.exec;
    }
    for (int launch = 0;; launch++) {
      if (launch > 0) {          // a new set of tags: stale reservations cleared
        EXH_CUDA_TRY(cudaMemsetAsync(h->resv, 0, sizeof(unsigned) * ng, st));
        EXH_CUDA_TRY(cudaMemsetAsync(dcnt + GROW_TAG, 0, sizeof(int), st));
      }
      EXH_CUDA_TRY(cudaGraphLaunch(ex, st));
      int tag = 0;
      EXH_CUDA_TRY(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
      EXH_CUDA_TRY(cudaMemcpyAsync(&tag, dcnt + GROW_TAG, sizeof(int), cudaMemcpyDeviceToHost, st));
      EXH_CUDA_TRY(cudaStreamSynchronize(st));
      count_launch(15 * (tag / 2));
      if (c.verbose > 1) {
        printf("  growth: %d rounds, %d left, %d growths in FP64\n", tag, hc[2], hc[GROW_NEXACT]);
        fflush(stdout);
      }
      if (hc[1] || hc[2] == 0) break;
      if ((size_t)launch * GROW_ROUNDS_PER_LAUNCH > (size_t)nproc + 2) {
        exh_set_error_msg("halo growth made no progress", __FILE__, __LINE__);
        return EXH_E_TIMEOUT;
      }
    }
  }
  if (hc[1]) {
    exh_set_error_msg(hc[1] == 1 ? "a halo grew past the sigma(M) table (find_halos.c:316 would read past Sig_Grid)"
                                 : "a halo grew past every shell of the box",
                      __FILE__, __LINE__);
    return EXH_E_RANGE;
  }
  if (timing_on()) {
    // algorithmic bytes of the growth rounds: one reduction over the peaks
    unsigned long long* dsum = reinterpret_cast<unsigned long long*>(dcnt + 6);   // 8-byte aligned slot
    EXH_CUDA_TRY(cudaMemsetAsync(dsum, 0, sizeof(unsigned long long), st));
    k_sum_words<<<EXH_NUM_SMS, 256, 0, st>>>(h->words, (int)nproc, dsum);
    count_launch(1);
    unsigned long long nw = 0;
    EXH_CUDA_TRY(cudaMemcpyAsync(&nw, dsum, sizeof(nw), cudaMemcpyDeviceToHost, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));
    kt.bytes = 4.0 * (double)nw;
  }
  k_kept<<<nb, 128, 0, st>>>(h->cnt, h->state, (int)nproc, hs.Nmin, kept);
  count_launch(1);
  int* total = dcnt + 2;
  // gfree is dead after the rounds: it serves as the scan's block sums
  EXH_CUDA_TRY(exclusive_scan<int>(kept, misc, nproc, h->gfree, total, st));
  int nh = 0;
  EXH_CUDA_TRY(cudaMemcpyAsync(&nh, total, sizeof(int), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  k_halo_index<<<nb, 128, 0, st>>>(kept, misc, (int)nproc, h->hid, h->hpeak);
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  h->nh = nh;
  return EXH_OK;
}

// ------------------------------------------------------------------ flags
__global__ void k_flags_ref(const int* __restrict__ flag, const int* __restrict__ hid, size_t ng,
                            long long* __restrict__ out) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < ng; i += stride) {
    const int v = flag[i];
    long long o;
    if (v == FLAG_FREE) o = (long long)ng;
    else if (v >= 0) o = hid[v] >= 0 ? (long long)hid[v] : (long long)ng + 1;
    else o = hid[-v - 2] >= 0 ? -(long long)hid[-v - 2] : (long long)ng + 1;
    out[i] = o;
  }
}

int flags_to_reference(const HaloDev& h, size_t ng, int64_t* out_dev, cudaStream_t st) {
  k_flags_ref<<<EXH_NUM_SMS * 8, 256, 0, st>>>(h.flag, h.hid, ng, reinterpret_cast<long long*>(out_dev));
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  return EXH_OK;
}

// ------------------------------------------------------------------ masses
// Compute_Mass (find_halos.c:455-476): halo h takes the h-th draw of the
// taus stream seeded with the seed; its mass interpolates I(M) between the
// member count and the next sphere count and inverts I.  Everything that
// depends on the count alone is tabulated on the host once per set of tables
// (same double operations as the per-halo evaluation): I at every sphere
// count, the first sphere-table entry of every count, and the inverse
// spline's interval coefficients.
constexpr int MASS_CHUNK = 8;

struct MassTables {
  const double* Itab;     // I(count * Mcell) per sphere-table entry, NaN outside the spline
  const int* first;       // count -> first sphere-table entry with that count (< min(nsph, Ncells)), or -1
  int nsph, Ncells;
  DevSplineCoef inv;      // M(I)
};

__global__ void k_masses(const TausJump* __restrict__ J, TausState s0, MassTables T, const int* __restrict__ hpeak,
                         const int* __restrict__ cnt, const unsigned* __restrict__ pid, int64_t np, int64_t nh,
                         HaloScalars hs, float* __restrict__ Mh, int* __restrict__ count_out, int* __restrict__ xc,
                         int* __restrict__ err) {
  const int64_t h0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * MASS_CHUNK;
  if (h0 >= nh) return;
  // state after h0 draws
  unsigned s[3] = {s0.s[0], s0.s[1], s0.s[2]};
  taus_jump(J, s, (unsigned long long)h0);
  const int64_t h1 = min(nh, h0 + MASS_CHUNK);
  int bad = 0;
  for (int64_t h = h0; h < h1; h++) {
    const double u = taus_u01(taus_next(s));
    const int r = hpeak[h];
    const int count = cnt[r];
    // Next_Count (find_halos.c:442-452): the first table entry equal to
    // count, and the entry after it
    const int lo = (count >= 0 && count <= T.Ncells) ? __ldg(&T.first[count]) : -1;
    float m = __int_as_float(0x7fc00000);
    if (lo < 0 || lo + 1 >= T.nsph) {
      bad = 1;
    } else {
      const double i0 = __ldg(&T.Itab[lo]), i1 = __ldg(&T.Itab[lo + 1]);
      if (isnan(i0) || isnan(i1)) {
        bad = 1;
      } else {
        const float dt = (float)__dadd_rn(i0, __dmul_rn(__dsub_rn(i1, i0), u));
        m = (float)T.inv.eval((double)dt, &bad);
      }
    }
    Mh[h] = m;
    count_out[h] = count;
    int x, y, z;
    peak_coords(pid[np - 1 - r], hs, x, y, z);
    xc[3 * h] = x; xc[3 * h + 1] = y; xc[3 * h + 2] = z;
  }
  if (bad) atomicExch(err, 1);
}

int halo_masses(Ctx& c, const BoxParams& b, const HaloDev& h, const HostTables& tab, float* Mh_dev, int* count_dev,
                int* xc_dev, cudaStream_t st) {
  if (h.nh == 0) return EXH_OK;
  // built once per process; the initialisation of a local static is thread-safe
  const TausJump& J = taus_jump_host();
  TausState s0;
  taus_seed_state((unsigned long)b.seed, s0.s);
  const std::vector<int>& sph = cells_in_spheres();
  const int Nr = tab.Nr, nsph = (int)sph.size(), Ncells = tab.Ncells;
  const size_t dbl = 5 * (size_t)Nr + nsph;
  const size_t bytes = sizeof(TausJump) + 16 + sizeof(double) * dbl + sizeof(int) * ((size_t)Ncells + 1) + 64;
  // device copies of the jump matrices and the count tables: uploaded once
  // per distinct set of tables and cell mass
  std::string key(reinterpret_cast<const char*>(tab.M.data()), sizeof(double) * Nr);
  key.append(reinterpret_cast<const char*>(tab.Int.data()), sizeof(double) * Nr);
  key.append(reinterpret_cast<const char*>(&b.Mcell), sizeof(float));
  key.append(reinterpret_cast<const char*>(&Ncells), sizeof(int));
  const bool cached = key == c.mass_key && c.buf[B_WORK2].p && c.buf[B_WORK2].cap >= bytes;
  if (!cached) c.mass_key.clear();
  EXH_TRY(c.buf[B_WORK2].ensure(bytes));
  char* base = c.buf[B_WORK2].as<char>();
  TausJump* dJ = reinterpret_cast<TausJump*>(base);
  double* dd = reinterpret_cast<double*>(base + ((sizeof(TausJump) + 15) & ~size_t(15)));
  int* dfirst = reinterpret_cast<int*>(dd + dbl);
  if (!cached) {
    Spline sI, sInv;
    if (sI.init(tab.M.data(), tab.Int.data(), Nr) != EXH_OK || sInv.init(tab.Int.data(), tab.M.data(), Nr) != EXH_OK) {
      exh_set_error_msg("mass-function integral is not increasing", __FILE__, __LINE__);
      return EXH_E_RANGE;
    }
    std::vector<double> hd(dbl);
    std::memcpy(&hd[0], sInv.x.data(), sizeof(double) * Nr);
    std::memcpy(&hd[Nr], sInv.y.data(), sizeof(double) * Nr);
    std::memcpy(&hd[2 * Nr], sInv.c.data(), sizeof(double) * Nr);
    for (int i = 0; i + 1 < Nr; i++) {       // Spline::eval's bb and dd of interval i
      const double xl = sInv.x[i], dx = sInv.x[i + 1] - xl, dy = sInv.y[i + 1] - sInv.y[i];
      const double c0 = sInv.c[i], c1 = sInv.c[i + 1];
      hd[3 * Nr + i] = dy / dx - dx * (c1 + 2.0 * c0) / 3.0;
      hd[4 * Nr + i] = (c1 - c0) / (3.0 * dx);
    }
    hd[4 * Nr - 1] = 0.0;
    hd[5 * Nr - 1] = 0.0;
    for (int j = 0; j < nsph; j++) {         // I at each sphere count, as m0 / m1 of the reference
      int bad = 0;
      const float m = (float)sph[j] * b.Mcell;
      const double v = sI.eval((double)m, &bad);
      hd[5 * Nr + j] = bad ? NAN : v;
    }
    std::vector<int> first((size_t)Ncells + 1, -1);
    for (int j = std::min(nsph, Ncells) - 1; j >= 0; j--)
      if (sph[j] >= 0 && sph[j] <= Ncells) first[sph[j]] = j;
    EXH_CUDA_TRY(cudaMemcpyAsync(dJ, &J, sizeof(J), cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaMemcpyAsync(dd, hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaMemcpyAsync(dfirst, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice, st));
    EXH_CUDA_TRY(cudaStreamSynchronize(st));   // the host vectors die here
    c.mass_key = key;
  }
  MassTables T;
  T.Itab = dd + 5 * Nr;
  T.first = dfirst;
  T.nsph = nsph;
  T.Ncells = Ncells;
  T.inv = DevSplineCoef{dd, dd + Nr, dd + 2 * Nr, dd + 3 * Nr, dd + 4 * Nr, Nr};
  EXH_TRY(c.buf[B_HOSTIO2].ensure(64));
  int* derr = c.buf[B_HOSTIO2].as<int>();
  EXH_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), st));
  HaloScalars hs{};
  hs.n0 = b.nd[0]; hs.n1 = b.nd[1]; hs.n2 = b.nd[2];
  const int64_t nchunk = (h.nh + MASS_CHUNK - 1) / MASS_CHUNK;
  { KTimer kt(KC_MASS, st, 0.0);
  k_masses<<<exh_div_up(nchunk, 128), 128, 0, st>>>(dJ, s0, T, h.hpeak, h.cnt, h.id, h.np, h.nh, hs, Mh_dev,
                                                   count_dev, xc_dev, derr); }
  count_launch(1);
  EXH_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  EXH_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  EXH_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    exh_set_error_msg("halo mass outside the mass-function tables", __FILE__, __LINE__);
    return EXH_E_RANGE;
  }
  return EXH_OK;
}

}  // namespace exh
