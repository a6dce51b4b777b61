// Aggregation AMG preconditioner for the batched solver, set up on the GPU
// (the sm_103a counterpart of gpu/src/amg.rs:127-773 and precond.rs:439-498).
//
// Hierarchy.  Every level is one packed block-diagonal CSR over all charts (chart rows stay
// contiguous, so aggregates never cross charts).  Per level and for every chart that is
// still coarsening:
//   * aggregation: two rounds of pairwise matching on |A| (each unmatched row proposes to
//     one of its strongly coupled unmatched neighbours, picked by a symmetric pseudo-random
//     pair priority; mutual proposals pair up), first on rows, then on the pairs ->
//     aggregates of about 4 rows (the reference's size-4 target, amg.rs:245, with a parallel
//     matching in place of its sequential scan);
//   * prolongator: tentative (one 1 per row, Precond::Amg) or smoothed
//     P = (I - omega D^-1 A) P_tent, omega = 2/3 (Precond::AmgSa, amg.rs:299-362);
//   * Galerkin operator A_c = R (A P), R = P^T (amg.rs:384-429), each product row formed by
//     a bounded, order-fixed accumulation (deterministic: no float atomics anywhere).
// A chart stops coarsening once it has <= kDirect rows (or its aggregation stalls); its
// last operator is factored densely (Cholesky, FP64 pivots, FP32 factor) by one CTA per
// chart, the batched counterpart of the reference's exact coarse factor (amg.rs:46-50).
//
// Apply (one V(1,1) cycle, z = M^-1 r, FP32): down: x = w D^-1 b, t = b - A x (one fused
// pass), b_c = R t; direct solves of every chart at its own last level (one CTA per chart);
// up: x += P x_c, x' = x + w D^-1 (b - A x).  Charts whose CG has converged are skipped.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>

#include "system.cuh"

namespace ruv {
namespace {

constexpr int kAmgThreads = 256;
constexpr int kDirect = 64;       // rows at which a chart is solved directly
constexpr int kMaxLevels = 16;
constexpr float kOmega = 2.0f / 3.0f;
// proposal rounds of each matching pass: 3 against 4 cost one CG iteration more at most and
// save about 2.3 ms of set-up on the 4096-disk step and 11 ms on the 2048^2 field's step
// (fewer iterations there too: 130 against 138)
constexpr int kPairRounds = 3;
// distinct keys per accumulated strength row: group strengths beyond it (only on dense coarse
// levels of the smoothed hierarchy) are left out of the matching, deterministically
constexpr int kAccCap = 48;
// Smoothed prolongator row cap (own aggregate always kept).  The reference keeps 32
// (amg.rs:299); on the device the cap sets the density of every coarse operator and so the
// set-up and V-cycle cost, and 4 gives the shortest whole solve (iterations nearly those of 8)
constexpr int kPMaxRow = 4;
// Levels with a smoothed prolongator in AMG-SA, tentative below: the coarse operators of a
// fully smoothed hierarchy are the densest, and two smoothed levels give the shortest solve on
// the measured workloads (4096 disks: 91.7 ms against 91.3 with all levels smoothed; the 2048^2
// height field: 129 ms against 180 with all, 146 with plain aggregation)
constexpr int kSaLevels = 2;
// Rows per CTA tile in the V-cycle kernels: 2048 on level 0, 512 on the coarser levels.  On
// the 4096 disks (step, 8 steps per setting, 1024 everywhere = 92.45 ms): level 0 at 2048
// -0.44 ms, at 512 +1.7 ms; levels 1-3 at 512 -0.88 ms, at 256 -0.58 ms, at 2048 +1.1 ms;
// level 0 at 2048 with levels 1-3 at 256 -1.02 ms.  Smaller coarse tiles spread the coarse
// levels' few rows per chart over more SMs; level 0 keeps its rows streaming longer per CTA.
constexpr int64_t kLevelTile0 = 2048, kLevelTile = 512;

// The k-th entry of the per-level list in the environment variable `knob` (entries separated
// by ',' or '/'), or 0 where the variable or its k-th entry is missing.
long long env_level_entry(const char* knob, int k) {
  const char* e = std::getenv(knob);
  if (!e) return 0;
  int i = 0;
  for (const char* q = e; *q; ++i) {
    if (i == k) return std::atoll(q);
    while (*q && *q != ',' && *q != '/') ++q;
    if (*q) ++q;
  }
  return 0;
}

// Rows per V-cycle tile of level k: the k-th entry of RUV_AMG_TILE (0 or missing: the default
// above; 64 to 65536 taken).
int64_t level_tile_rows(int k) {
  const long long v = env_level_entry("RUV_AMG_TILE", k);
  if (v >= 64 && v <= 65536) return v;
  return k == 0 ? kLevelTile0 : kLevelTile;
}

__device__ __forceinline__ int64_t find_chart64(const int64_t* off, int64_t n_charts, int64_t i) {
  int64_t lo = 0, hi = n_charts;
  while (hi - lo > 1) {
    int64_t mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// Bounded accumulation of (key, value) products in arrival order; keys sorted at the end.
template <int CAP, class T = float>
struct Acc {
  int key[CAP];
  T val[CAP];
  int n = 0;
  bool overflow = false;
  __device__ __forceinline__ void add(int k, T v) {
    for (int t = 0; t < n; ++t)
      if (key[t] == k) {
        val[t] += v;
        return;
      }
    if (n < CAP) {
      key[n] = k;
      val[n] = v;
      ++n;
    } else {
      overflow = true;
    }
  }
  __device__ __forceinline__ void sort() {
    for (int i = 1; i < n; ++i) {
      int k = key[i];
      T v = val[i];
      int j = i - 1;
      while (j >= 0 && key[j] > k) {
        key[j + 1] = key[j];
        val[j + 1] = val[j];
        --j;
      }
      key[j + 1] = k;
      val[j + 1] = v;
    }
  }
};

// max of v over the active lanes, one atomic per warp (a statistic, read in debug output)
__device__ __forceinline__ void warp_atomic_max(int* p, int v) {
  const unsigned m = __activemask();
  const int w = __reduce_max_sync(m, v);
  if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicMax(p, w);
}

// ---------------------------------------------------------------- setup kernels
// Row -> chart and whether the chart keeps coarsening at this level.
__global__ void k_row_chart(int64_t n, const int64_t* __restrict__ chart_row, int64_t n_charts,
                            const int32_t* __restrict__ cont, int32_t* __restrict__ row_chart,
                            uint8_t* __restrict__ active) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t c = find_chart64(chart_row, n_charts, i);
  row_chart[i] = (int32_t)c;
  active[i] = cont[c] ? 1 : 0;
}

// Symmetric pseudo-random priority of the pair {i, j} (a 64-bit mix of the ordered pair).
__device__ __forceinline__ uint32_t pair_priority(int32_t i, int32_t j) {
  uint64_t x = ((uint64_t)(uint32_t)min(i, j) << 32) | (uint32_t)max(i, j);
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return (uint32_t)x;
}

// Pairwise matching, proposal: among the unmatched neighbours coupled at least kStrong times
// as strongly as the strongest one, the one of highest pair priority (ties to the smaller j).
// Choosing by a symmetric random priority rather than by the coupling itself makes mutual
// proposals likely even where couplings vary monotonically along a row of the mesh (a
// weight-ordered handshake then chains i -> i-1 -> i-2 ... and pairs almost nothing).
constexpr float kStrong = 0.85f;
__global__ void k_propose(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                          const float* __restrict__ vals, const uint8_t* __restrict__ active,
                          const int32_t* __restrict__ mate, int32_t* __restrict__ prop, float strong) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t best = -1;
  if (active[i] && mate[i] < 0) {
    float mx = 0.0f;
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int32_t j = cols[e];
      if (j != i && mate[j] < 0) mx = fmaxf(mx, fabsf(vals[e]));
    }
    uint32_t bp = 0;
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int32_t j = cols[e];
      if (j == i || mate[j] >= 0 || !(fabsf(vals[e]) >= strong * mx) || mx == 0.0f) continue;
      const uint32_t pr = pair_priority((int32_t)i, j);
      if (best < 0 || pr > bp || (pr == bp && j < best)) {
        bp = pr;
        best = j;
      }
    }
  }
  prop[i] = best;
}

__global__ void k_accept(int64_t n, const int32_t* __restrict__ prop, int32_t* __restrict__ mate) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t j = prop[i];
  if (j > i && prop[j] == (int32_t)i) {
    mate[i] = j;
    mate[j] = (int32_t)i;
  }
}

// Lead row of each active row after pairing: its pair's smaller row; an unmatched row joins
// the pair of its strongest matched neighbour (|a_ij|, ties to the smaller j), or stays
// alone when it has none.  Every row ends in a group, so coarsening cannot stall.
__global__ void k_row_lead(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                           const float* __restrict__ vals, const uint8_t* __restrict__ active,
                           const int32_t* __restrict__ mate, int32_t* __restrict__ lead_row, uint8_t* __restrict__ lead) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!active[i]) {
    lead[i] = 0;
    return;
  }
  int32_t L;
  if (mate[i] >= 0) {
    L = min((int32_t)i, mate[i]);
  } else {
    int32_t best = -1;
    float bs = -1.0f;
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int32_t j = cols[e];
      if (j == i || mate[j] < 0) continue;
      const float sj = fabsf(vals[e]);
      if (sj > bs || (sj == bs && j < best)) {
        bs = sj;
        best = j;
      }
    }
    L = best >= 0 ? min(best, mate[best]) : (int32_t)i;
  }
  lead_row[i] = L;
  lead[i] = L == (int32_t)i ? 1 : 0;
}

__global__ void k_group_of(int64_t n, const uint8_t* __restrict__ active, const int32_t* __restrict__ lead_row,
                           const int64_t* __restrict__ gid, int32_t* __restrict__ grp_of, int32_t* __restrict__ gcnt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !active[i]) return;
  const int32_t g = (int32_t)gid[lead_row[i]];
  grp_of[i] = g;
  atomicAdd(&gcnt[g], 1);
}

__global__ void k_group_scatter(int64_t n, const uint8_t* __restrict__ active, const int32_t* __restrict__ grp_of,
                                const int64_t* __restrict__ goff, int32_t* __restrict__ cursor, int32_t* __restrict__ mem) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !active[i]) return;
  const int32_t g = grp_of[i];
  mem[goff[g] + atomicAdd(&cursor[g], 1)] = (int32_t)i;
}

__global__ void k_sort_members(int64_t ng, const int64_t* __restrict__ goff, int32_t* __restrict__ mem) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  for (int64_t a = goff[g] + 1; a < goff[g + 1]; ++a) {
    int32_t k = mem[a];
    int64_t j = a - 1;
    while (j >= goff[g] && mem[j] > k) {
      mem[j + 1] = mem[j];
      --j;
    }
    mem[j + 1] = k;
  }
}

// Strengths from group g to its neighbour groups (sum of |a| between members), in member
// and entry order.  Only groups passing `want(h)` are accumulated.
template <class Want>
__device__ __forceinline__ void group_strengths(int64_t g, const int64_t* goff, const int32_t* mem, const int32_t* rp,
                                                const int32_t* cols, const float* vals, const int32_t* grp_of,
                                                Acc<kAccCap>& acc, Want want) {
  for (int64_t a = goff[g]; a < goff[g + 1]; ++a) {
    const int32_t i = mem[a];
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int32_t h = grp_of[cols[e]];
      if (h == (int32_t)g || !want(h)) continue;
      acc.add(h, fabsf(vals[e]));
    }
  }
}

// Second matching level, on groups: propose to a strongly coupled unmatched neighbour group.
__global__ void k_propose2(int64_t ng, const int64_t* __restrict__ goff, const int32_t* __restrict__ mem,
                           const int32_t* __restrict__ rp, const int32_t* __restrict__ cols, const float* __restrict__ vals,
                           const int32_t* __restrict__ grp_of, const int32_t* __restrict__ gmate,
                           int32_t* __restrict__ prop, int* __restrict__ stats, float strong) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int32_t best = -1;
  if (gmate[g] < 0) {
    Acc<kAccCap> acc;
    group_strengths(g, goff, mem, rp, cols, vals, grp_of, acc, [&](int32_t h) { return gmate[h] < 0; });
    warp_atomic_max(stats + 2, acc.n);
    float mx = 0.0f;
    for (int t = 0; t < acc.n; ++t) mx = fmaxf(mx, acc.val[t]);
    uint32_t bp = 0;
    for (int t = 0; t < acc.n; ++t) {  // as k_propose, on groups
      if (!(acc.val[t] >= strong * mx) || mx == 0.0f) continue;
      const uint32_t pr = pair_priority((int32_t)g, acc.key[t]);
      if (best < 0 || pr > bp || (pr == bp && acc.key[t] < best)) {
        bp = pr;
        best = acc.key[t];
      }
    }
  }
  prop[g] = best;
}

// The group graph of a level, built once for all matching rounds: per group g, its
// neighbour groups h != g with the summed |a_ij| between their members, the keys in order of
// first arrival (members in order, entries in order) and each sum in arrival order -- what
// group_strengths accumulates, for every key.  A round then filters the stored row (the
// first kAccCap wanted keys in arrival order are exactly the ones the bounded accumulator
// keeps), so the matching is the same bit for bit.  Row g lives at gcap_off[g] (room for
// the members' entries) with gn[g] keys.
__global__ void k_group_nnz(int64_t ng, const int64_t* __restrict__ goff, const int32_t* __restrict__ mem,
                            const int32_t* __restrict__ rp, int32_t* __restrict__ gcap) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int32_t c = 0;
  for (int64_t a = goff[g]; a < goff[g + 1]; ++a) c += rp[mem[a] + 1] - rp[mem[a]];
  gcap[g] = c;
}
__global__ void k_group_graph(int64_t ng, const int64_t* __restrict__ goff, const int32_t* __restrict__ mem,
                              const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                              const float* __restrict__ vals, const int32_t* __restrict__ grp_of,
                              const int64_t* __restrict__ gcap_off, int32_t* __restrict__ gn, int32_t* __restrict__ gkey,
                              float* __restrict__ gval) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int32_t* K = gkey + gcap_off[g];
  float* V = gval + gcap_off[g];
  // the first kReg keys in registers (every index a compile-time constant once unrolled), the
  // rest in the row's global area; each key's strength summed in entry order
  constexpr int kReg = 16;
  int32_t rk[kReg];
  float rv[kReg];
#pragma unroll
  for (int t = 0; t < kReg; ++t) {
    rk[t] = -1;
    rv[t] = 0.0f;
  }
  int n = 0;
  for (int64_t a = goff[g]; a < goff[g + 1]; ++a) {
    const int32_t i = mem[a];
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int32_t h = grp_of[cols[e]];
      if (h == (int32_t)g) continue;
      const float v = fabsf(vals[e]);
      bool hit = false;
#pragma unroll
      for (int t = 0; t < kReg; ++t)
        if (rk[t] == h) {  // (unused slots hold -1, never a group)
          rv[t] += v;
          hit = true;
        }
      if (hit) continue;
      int t = kReg;
      while (t < n && K[t] != h) ++t;
      if (t < n) {
        V[t] += v;
      } else if (n < kReg) {
#pragma unroll
        for (int q = 0; q < kReg; ++q)
          if (q == n) {
            rk[q] = h;
            rv[q] = v;
          }
        ++n;
      } else {
        K[n] = h;
        V[n] = v;
        ++n;
      }
    }
  }
#pragma unroll
  for (int t = 0; t < kReg; ++t)
    if (t < n) {
      K[t] = rk[t];
      V[t] = rv[t];
    }
  gn[g] = n;
}

// k_propose2 over the stored group graph.
__global__ void k_propose2_graph(int64_t ng, const int64_t* __restrict__ gcap_off, const int32_t* __restrict__ gn,
                                 const int32_t* __restrict__ gkey, const float* __restrict__ gval,
                                 const int32_t* __restrict__ gmate, int32_t* __restrict__ prop, int* __restrict__ stats,
                                 float strong) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int32_t best = -1;
  if (gmate[g] < 0) {
    const int32_t* K = gkey + gcap_off[g];
    const float* V = gval + gcap_off[g];
    const int n = gn[g];
    float mx = 0.0f;
    int kept = 0, t_end = n;
    for (int t = 0; t < n; ++t) {
      if (gmate[K[t]] >= 0) continue;
      if (kept == kAccCap) {
        t_end = t;
        break;
      }
      ++kept;
      mx = fmaxf(mx, V[t]);
    }
    warp_atomic_max(stats + 2, kept);
    uint32_t bp = 0;
    for (int t = 0; t < t_end; ++t) {
      if (gmate[K[t]] >= 0) continue;
      if (!(V[t] >= strong * mx) || mx == 0.0f) continue;
      const uint32_t pr = pair_priority((int32_t)g, K[t]);
      if (best < 0 || pr > bp || (pr == bp && K[t] < best)) {
        bp = pr;
        best = K[t];
      }
    }
  }
  prop[g] = best;
}

// k_group_lead over the stored group graph.
__global__ void k_group_lead_graph(int64_t ng, const int64_t* __restrict__ gcap_off, const int32_t* __restrict__ gn,
                                   const int32_t* __restrict__ gkey, const float* __restrict__ gval,
                                   const int32_t* __restrict__ gmate, int32_t* __restrict__ glead_of,
                                   uint8_t* __restrict__ glead) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int32_t L;
  if (gmate[g] >= 0) {
    L = min((int32_t)g, gmate[g]);
  } else {
    const int32_t* K = gkey + gcap_off[g];
    const float* V = gval + gcap_off[g];
    const int n = gn[g];
    int32_t best = -1;
    float bs = -1.0f;
    int kept = 0;
    for (int t = 0; t < n && kept < kAccCap; ++t) {
      if (gmate[K[t]] < 0) continue;
      ++kept;
      if (V[t] > bs || (V[t] == bs && K[t] < best)) {
        bs = V[t];
        best = K[t];
      }
    }
    L = best >= 0 ? min(best, gmate[best]) : (int32_t)g;
  }
  glead_of[g] = L;
  glead[g] = L == (int32_t)g ? 1 : 0;
}

// Lead group of each group after pairing groups (unmatched groups join the pair of their
// strongest matched neighbour group).
__global__ void k_group_lead(int64_t ng, const int64_t* __restrict__ goff, const int32_t* __restrict__ mem,
                             const int32_t* __restrict__ rp, const int32_t* __restrict__ cols, const float* __restrict__ vals,
                             const int32_t* __restrict__ grp_of, const int32_t* __restrict__ gmate,
                             int32_t* __restrict__ glead_of, uint8_t* __restrict__ glead) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int32_t L;
  if (gmate[g] >= 0) {
    L = min((int32_t)g, gmate[g]);
  } else {
    Acc<kAccCap> acc;
    group_strengths(g, goff, mem, rp, cols, vals, grp_of, acc, [&](int32_t h) { return gmate[h] >= 0; });
    int32_t best = -1;
    float bs = -1.0f;
    for (int t = 0; t < acc.n; ++t)
      if (acc.val[t] > bs || (acc.val[t] == bs && acc.key[t] < best)) {
        bs = acc.val[t];
        best = acc.key[t];
      }
    L = best >= 0 ? min(best, gmate[best]) : (int32_t)g;
  }
  glead_of[g] = L;
  glead[g] = L == (int32_t)g ? 1 : 0;
}

// agg[i] = coarse row of row i (aggregates numbered in lead-group order).
__global__ void k_agg(int64_t n, const uint8_t* __restrict__ active, const int32_t* __restrict__ grp_of,
                      const int32_t* __restrict__ glead_of, const int64_t* __restrict__ aid, int32_t* __restrict__ agg) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  agg[i] = active[i] ? (int32_t)aid[glead_of[grp_of[i]]] : -1;
}

// Prolongator rows.  MODE 0: count, MODE 1: fill.  Tentative: one 1 at agg[i].  Smoothed:
// row i = e_agg[i] - w/d_i * sum_j a_ij e_agg[j] (amg.rs:308-362), truncated to its kPMaxRow
// largest entries with the own aggregate always kept (amg.rs:331-356), keys ascending.
template <int MODE>
__global__ void k_prolong(int64_t n, const uint8_t* __restrict__ active, const int32_t* __restrict__ rp,
                          const int32_t* __restrict__ cols, const float* __restrict__ vals,
                          const float* __restrict__ dinv, const int32_t* __restrict__ agg, int smooth, int pmax,
                          int32_t* __restrict__ cnt, const int64_t* __restrict__ off, int32_t* __restrict__ pc,
                          float* __restrict__ pv, int* __restrict__ overflow) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!active[i]) {
    if (MODE != 1) cnt[i] = 0;
    return;
  }
  Acc<kAccCap> acc;
  acc.add(agg[i], 1.0f);
  if (smooth) {
    const float wd = kOmega * dinv[i];
    for (int e = rp[i]; e < rp[i + 1]; ++e) acc.add(agg[cols[e]], -wd * vals[e]);
    if (acc.n > pmax) {
      // keep the own aggregate (slot 0) and the pmax - 1 largest magnitudes (ties to the
      // smaller column): selection by repeated maximum, then compaction
      bool keep[kAccCap];
      for (int t = 0; t < acc.n; ++t) keep[t] = t == 0;
      for (int k = 1; k < pmax; ++k) {
        int bt = -1;
        for (int t = 1; t < acc.n; ++t) {
          if (keep[t]) continue;
          if (bt < 0 || fabsf(acc.val[t]) > fabsf(acc.val[bt]) ||
              (fabsf(acc.val[t]) == fabsf(acc.val[bt]) && acc.key[t] < acc.key[bt]))
            bt = t;
        }
        keep[bt] = true;
      }
      int m = 0;
      for (int t = 0; t < acc.n; ++t)
        if (keep[t]) {
          acc.key[m] = acc.key[t];
          acc.val[m] = acc.val[t];
          ++m;
        }
      acc.n = m;
    }
    acc.sort();
  }
  if (acc.overflow) atomicExch(overflow, 1);
  warp_atomic_max(overflow + 3, acc.n);
  if (MODE == 0) {
    cnt[i] = acc.n;
  } else if (MODE == 2) {  // counts and the row into a staging slot of pmax entries (off unused)
    cnt[i] = acc.n;
    const int64_t at = i * (int64_t)pmax;
    for (int t = 0; t < acc.n && t < pmax; ++t) {
      pc[at + t] = acc.key[t];
      pv[at + t] = acc.val[t];
    }
  } else {
    int64_t at = off[i];
    for (int t = 0; t < acc.n; ++t) {
      pc[at + t] = acc.key[t];
      pv[at + t] = acc.val[t];
    }
  }
}

// Staged prolongator rows (pmax slots each) to their CSR places.
__global__ void k_prolong_copy(int64_t n, int pmax, const int32_t* __restrict__ cnt, const int32_t* __restrict__ st_c,
                               const float* __restrict__ st_v, const int64_t* __restrict__ off, int32_t* __restrict__ pc,
                               float* __restrict__ pv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int m = cnt[i];
  const int64_t src = i * (int64_t)pmax, dst = off[i];
  for (int t = 0; t < m; ++t) {
    pc[dst + t] = st_c[src + t];
    pv[dst + t] = st_v[src + t];
  }
}

// Transpose (R = P^T): counts per coarse row, then a stable scatter by fine row order.
__global__ void k_count_cols(int64_t nnz, const int32_t* __restrict__ pc, int32_t* __restrict__ cnt) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nnz) atomicAdd(&cnt[pc[e]], 1);
}

__global__ void k_scatter_t(int64_t n, const int64_t* __restrict__ poff, const int32_t* __restrict__ pc,
                            const float* __restrict__ pv, const int64_t* __restrict__ roff,
                            int32_t* __restrict__ cursor, int32_t* __restrict__ rc, float* __restrict__ rv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t e = poff[i]; e < poff[i + 1]; ++e) {
    int32_t c = pc[e];
    int64_t at = roff[c] + atomicAdd(&cursor[c], 1);
    rc[at] = (int32_t)i;
    rv[at] = pv[e];
  }
}

// Each row of R ordered by fine row (a deterministic order after the atomic scatter): warp
// per row, every entry placed at the count of smaller keys (the keys of a row are distinct).
__global__ void k_sort_rows(int64_t n, const int64_t* __restrict__ off, const int32_t* __restrict__ c_in,
                            const float* __restrict__ v_in, int32_t* __restrict__ c, float* __restrict__ v) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= n) return;
  const int64_t b = off[r], e = off[r + 1];
  for (int64_t i0 = b; i0 < e; i0 += 32) {
    const int64_t i = i0 + lane;
    const int32_t k = i < e ? c_in[i] : INT32_MAX;
    int rank = 0;
    for (int64_t u0 = b; u0 < e; u0 += 32) {
      const int32_t ku = u0 + lane < e ? c_in[u0 + lane] : INT32_MAX;
      const int m = e - u0 < 32 ? (int)(e - u0) : 32;
      for (int u = 0; u < m; ++u) rank += __shfl_sync(kFull, ku, u) < k;
    }
    if (i < e) {
      c[b + rank] = k;
      v[b + rank] = v_in[i];
    }
  }
}

// ---------------------------------------------------------------- sparse products (Galerkin)
// Row `row` of a two-level product: for each outer entry q of the row (index j, scale s_q, in
// order) and each inner entry r of row j (in order), the product s_q * v_r under the key
// key(idx_r); equal keys summed in that arrival order.  W = A P (outer A, inner P),
// A_c = R W (outer R, inner W), and A_c = R A P_t for the tentative prolongator (outer R,
// inner A with keys through agg).  Output rows hold their keys ascending with the sums (DIAG:
// also the inverse of the entry on the diagonal).
//
// G lanes per row (32 / G rows per warp).  The lanes take G consecutive products at a time
// (the owner outer entry of each found by a binary search over the scanned inner lengths,
// so the inner loads are contiguous), insert the keys into the row's open-addressing table
// of H slots in shared memory, and the lowest lane of every group of equal keys adds the
// group's products to the slot in lane order -- the arrival order, so the sums are those of a
// sequential accumulator and deterministic.  The occupied slots are then compacted and each
// ranked by counting smaller keys.
//   MODE 2 (one evaluation): writes the row to a staging area of H/2 entries per row, or, if
//          it has more distinct keys, lists it (sn = -1) for the large-table kernel;
//   MODE 0 / 1: counts / writes at off[row] (the large-table kernel, rows from the list).
//
// Arithmetic: every operand and sum is a double-float pair (hi, lo: FP32 values whose sum
// carries about 48 significant bits), formed by error-free FP32 transformations on the FMA
// pipe.  GB300 issues FP64 at a small fraction of its FP32 rate, and with FP64 products and
// sums these kernels were bound by the FP64 pipe (78% busy); the products' relative error
// stays near 1e-14, far below what the FP32 V-cycle can see.  Operands come through loaders:
// FP32 values (P, R), (hi, lo) array pairs (a level's operator) or pair arrays (W).
struct KeyId {
  __device__ __forceinline__ int32_t operator()(int32_t k) const { return k; }
};
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float s = a.x + b.x;
  const float bb = s - a.x;
  const float err = (a.x - (s - bb)) + (b.x - bb);
  const float lo = err + a.y + b.y;
  const float h = s + lo;
  return make_float2(h, lo - (h - s));
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float h = p + e;
  return make_float2(h, e - (h - p));
}
struct LdOne {  // no values: every entry 1
  static constexpr bool kHas = false;
  __device__ __forceinline__ float2 operator()(int64_t) const { return make_float2(1.0f, 0.0f); }
};
struct LdF {  // FP32 values
  const float* v;
  static constexpr bool kHas = true;
  __device__ __forceinline__ float2 operator()(int64_t e) const { return make_float2(v[e], 0.0f); }
};
struct LdHL {  // a level operator: hi and lo halves in two arrays
  const float* h;
  const float* l;
  static constexpr bool kHas = true;
  __device__ __forceinline__ float2 operator()(int64_t e) const { return make_float2(h[e], l[e]); }
};
struct LdDF {  // pairs
  const float2* v;
  static constexpr bool kHas = true;
  __device__ __forceinline__ float2 operator()(int64_t e) const { return v[e]; }
};
struct KeyAgg {
  const int32_t* agg;
  __device__ __forceinline__ int32_t operator()(int32_t k) const { return agg[k]; }
};

template <int G, int H>
struct GalSmem {
  static constexpr int HS = H / 2;  // distinct keys a row may hold
  static constexpr size_t bytes = sizeof(float2) * (H + G) + sizeof(int32_t) * (H + 2 * HS);
};

struct GalOut {
  int32_t* cnt;         // distinct keys per row (MODE 0, 2)
  int32_t* sn;          // MODE 2: staged count, or -1 when listed
  int32_t* st_key;      // MODE 2: staging, H/2 entries per row
  float2* st_val;
  const int64_t* off;   // MODE 1: output offsets
  int32_t* oc;
  float2* ov;
  float* adinv;         // DIAG
  int32_t* next;        // MODE 2: listed rows
  int32_t* next_n;
  int* overflow;        // MODE 0 / 1: a row above the large table's capacity
};

template <int MODE, int G, int H, int WARPS, bool DIAG, class OP, class OL, class IP, class IL, class KeyF>
__global__ void __launch_bounds__(32 * WARPS) k_gal_hash(int64_t nrows, const int32_t* __restrict__ list,
                                                         const uint8_t* __restrict__ active, const OP* __restrict__ o_ptr,
                                                         const int32_t* __restrict__ o_idx, OL o_val,
                                                         const IP* __restrict__ i_ptr, const int32_t* __restrict__ i_idx,
                                                         IL i_val, KeyF keyf, GalOut out) {
  using S = GalSmem<G, H>;
  constexpr int HS = S::HS;
  constexpr int SUB = 32 / G;
  constexpr int LOGH = __builtin_ctz(H);
  static_assert((H & (H - 1)) == 0 && HS >= G, "table size");
  extern __shared__ __align__(16) unsigned char gal_smem[];
  const int lane = threadIdx.x & 31, sl = lane & (G - 1), gb = lane & ~(G - 1);
  const unsigned smask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << gb);
  const int sw = (threadIdx.x >> 5) * SUB + (lane / G);
  unsigned char* base = gal_smem + S::bytes * (size_t)sw;
  float2* tval = reinterpret_cast<float2*>(base);
  float2* stage = tval + H;
  int32_t* tkey = reinterpret_cast<int32_t*>(stage + G);
  int32_t* ckey = tkey + H;
  int32_t* cslot = ckey + HS;
  const int64_t nsub = (int64_t)gridDim.x * WARPS * SUB;
  // the table starts empty; every row leaves it empty (only its own slots are cleared)
  auto clear_all = [&]() {
    for (int t = sl; t < H; t += G) {
      tkey[t] = -1;
      tval[t] = make_float2(0.0f, 0.0f);
    }
    __syncwarp(smask);
  };
  clear_all();
  for (int64_t k0 = (int64_t)blockIdx.x * WARPS * SUB + sw; k0 < nrows; k0 += nsub) {
    const int64_t row = list ? (int64_t)list[k0] : k0;
    if (active && !active[row]) {
      if (sl == 0) {
        if (MODE != 1) out.cnt[row] = 0;
        if (MODE == 2) out.sn[row] = 0;
      }
      continue;
    }
    const int64_t ob = (int64_t)o_ptr[row], oe = (int64_t)o_ptr[row + 1];
    int d = 0;
    bool over = false;
    for (int64_t q0 = ob; q0 < oe && !over; q0 += G) {
      const int64_t q = q0 + sl;
      int64_t ib = 0;
      int len = 0;
      float2 sc = make_float2(0.0f, 0.0f);
      if (q < oe) {
        const int32_t j = o_idx[q];
        if (MODE != 0) sc = o_val(q);
        ib = (int64_t)i_ptr[j];
        len = (int)((int64_t)i_ptr[j + 1] - ib);
      }
      int x = len;  // inclusive scan of the inner lengths over the sub-warp
#pragma unroll
      for (int o = 1; o < G; o <<= 1) {
        const int y = __shfl_up_sync(smask, x, o, G);
        if (sl >= o) x += y;
      }
      const int total = __shfl_sync(smask, x, G - 1, G);
      for (int p0 = 0; p0 < total; p0 += G) {
        const int pl = p0 + sl;
        const bool valid = pl < total;
        int own = 0;  // lanes whose inclusive end is <= pl
#pragma unroll
        for (int st = G / 2; st >= 1; st >>= 1) {
          const int xv = __shfl_sync(smask, x, own + st - 1, G);
          if (xv <= pl) own += st;
        }
        own = min(own, G - 1);
        const float2 sco = make_float2(__shfl_sync(smask, sc.x, own, G), __shfl_sync(smask, sc.y, own, G));
        const long long ibo = __shfl_sync(smask, (long long)ib, own, G);
        const int sto = __shfl_sync(smask, x - len, own, G);
        int32_t key = 0;
        float2 v = make_float2(0.0f, 0.0f);
        int slot = -1;
        bool fresh = false;
        if (valid) {
          const int64_t e = (int64_t)ibo + (pl - sto);
          key = keyf(i_idx[e]);
          if (MODE != 0) v = df_mul(sco, i_val(e));
          unsigned h = ((uint32_t)key * 0x9E3779B1u) >> (32 - LOGH);
          for (int pr = 0; pr < H; ++pr) {
            const int32_t k = reinterpret_cast<volatile int32_t*>(tkey)[h];
            if (k == key) {
              slot = (int)h;
              break;
            }
            if (k == -1) {
              const int32_t old = atomicCAS(&tkey[h], -1, key);
              if (old == -1 || old == key) {
                slot = (int)h;
                fresh = old == -1;
                break;
              }
            }
            h = (h + 1) & (H - 1);
          }
        }
        const unsigned fm = __ballot_sync(smask, fresh);
        if (fresh) {  // the occupied slots in insertion order
          const int pos = d + __popc(fm & ((1u << lane) - 1u));
          if (pos < HS) {
            ckey[pos] = key;
            cslot[pos] = slot;
          }
        }
        d += __popc(fm);
        if (__ballot_sync(smask, valid && slot < 0) != 0u || d > HS) {
          over = true;
          break;
        }
        if (MODE != 0) {
          stage[sl] = v;
          __syncwarp(smask);
          const unsigned gm = __match_any_sync(smask, valid ? slot : -1);
          if (valid && (__ffs(gm) - 1) == lane) {
            float2 s = tval[slot];
            for (unsigned m = gm; m != 0u; m &= m - 1u) s = df_add(s, stage[(__ffs(m) - 1) - gb]);
            tval[slot] = s;
          }
        }
        __syncwarp(smask);
      }
    }
    if (over) {
      if (sl == 0) {
        if (MODE == 2) {
          out.sn[row] = -1;
          out.cnt[row] = 0;
          out.next[atomicAdd(out.next_n, 1)] = (int32_t)row;
        } else {
          atomicExch(out.overflow, 1);
          if (MODE == 0) out.cnt[row] = 0;
        }
      }
      __syncwarp(smask);
      clear_all();
      continue;
    }
    __syncwarp(smask);
    if (MODE == 0) {
      if (sl == 0) out.cnt[row] = d;
      for (int c = sl; c < d; c += G) tkey[cslot[c]] = -1;
      __syncwarp(smask);
      continue;
    }
    // rank each key by counting smaller ones
    int32_t* dk;
    float2* dv;
    if (MODE == 2) {
      dk = out.st_key + row * HS;
      dv = out.st_val + row * HS;
    } else {
      dk = out.oc + out.off[row];
      dv = out.ov + out.off[row];
    }
    bool has_d = false;
    float dval = 0.0f;
    for (int c = sl; c < d; c += G) {
      const int32_t k = ckey[c];
      int rank = 0;
      for (int u = 0; u < d; ++u) rank += ckey[u] < k;
      const int slot = cslot[c];
      const float2 val = tval[slot];
      dk[rank] = k;
      dv[rank] = val;
      if (DIAG && k == (int32_t)row) {
        has_d = true;
        dval = val.x;
      }
    }
    if (DIAG) {
      if (__ballot_sync(smask, has_d) == 0u) {
        if (sl == 0) out.adinv[row] = 0.0f;
      } else if (has_d) {
        out.adinv[row] = dval > 0.0f ? 1.0f / dval : 0.0f;  // (hi of a normalised pair: lo changes no FP32 bit)
      }
    }
    if (MODE == 2 && sl == 0) {  // (MODE 1 leaves the counts alone)
      out.cnt[row] = d;
      out.sn[row] = d;
    }
    __syncwarp(smask);
    for (int c = sl; c < d; c += G) {
      const int slot = cslot[c];
      tkey[slot] = -1;
      tval[slot] = make_float2(0.0f, 0.0f);
    }
    __syncwarp(smask);
  }
}

// Staged rows to their place in the product (8 lanes per row); listed rows (sn < 0) are
// written by the large-table kernel.
__global__ void k_gal_copy(int64_t nrows, int hs, const int32_t* __restrict__ sn, const int32_t* __restrict__ st_key,
                           const float2* __restrict__ st_val, const int64_t* __restrict__ off, int32_t* __restrict__ oc,
                           float2* __restrict__ ov) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = t >> 3;
  const int sl = (int)(t & 7);
  if (row >= nrows) return;
  const int n = sn[row];
  const int64_t src = row * hs, dst = off[row];
  for (int k = sl; k < n; k += 8) {
    oc[dst + k] = st_key[src + k];
    ov[dst + k] = st_val[src + k];
  }
}

__global__ void k_i64_i32(int64_t n, const int64_t* __restrict__ a, int32_t* __restrict__ b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (int32_t)a[i];
}

// A coarse operator's pairs into its FP32 values (hi), their low halves and FP64 values.
__global__ void k_df_unpack(int64_t n, const float2* __restrict__ v, float* __restrict__ hi, float* __restrict__ lo,
                            double* __restrict__ v64) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 a = v[i];
  hi[i] = a.x;
  lo[i] = a.y;
  v64[i] = (double)a.x + (double)a.y;
}

// lo = (float)(v - hi) for an operator whose FP32 values hi = (float)v are given
__global__ void k_lo_half(int64_t n, const double* __restrict__ v, const float* __restrict__ hi, float* __restrict__ lo) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lo[i] = (float)(v[i] - (double)hi[i]);
}


__global__ void k_f64_f32_inv(int64_t n, const double* __restrict__ d, float* __restrict__ inv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) inv[i] = d[i] != 0.0 ? (float)(1.0 / d[i]) : 0.0f;
}

// Coarse chart offsets: chart_row_c[c] = aid at the chart's first row (aggregates are
// numbered in row order, per chart contiguous).
__global__ void k_coarse_chart_rows(int64_t n_charts, const int64_t* __restrict__ chart_row,
                                    const int64_t* __restrict__ lead_scan_rows, int64_t* __restrict__ out) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c <= n_charts) out[c] = lead_scan_rows[chart_row[c]];
}

// Row i heads an aggregate iff it leads its group and that group leads its aggregate
// (`lead` is 0 for inactive rows, so grp_of is only read for active ones).
__global__ void k_agg_lead_rows(int64_t n, const uint8_t* __restrict__ lead, const uint8_t* __restrict__ glead,
                                const int32_t* __restrict__ grp_of, uint8_t* __restrict__ arow) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) arow[i] = (lead[i] && glead[grp_of[i]]) ? 1 : 0;
}

// Dense inverse of each final chart block (<= kDirect rows), one CTA per chart, in shared
// memory: Cholesky A = L L^T, then Y = L^-1, then A^-1 = Y^T Y, stored as FP32 (symmetric,
// row-major m x m).  The V-cycle's coarse solve is then one dense mat-vec per chart instead
// of two serial triangular sweeps.
constexpr int kFactorThreads = 128;
constexpr size_t kFactorSmem = 2 * sizeof(float2) * kDirect * kDirect;

// df helpers of the dense factors: a - b, a / b and sqrt(a) on (hi, lo) pairs (one Newton
// correction each on the FP32 quotient / root, the residual formed with error-free products)
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_div(float2 a, float2 b) {
  const float q1 = a.x / b.x;
  const float2 r = df_add(a, df_neg(df_mul(make_float2(q1, 0.0f), b)));
  const float q2 = r.x / b.x;
  return df_add(make_float2(q1, 0.0f), make_float2(q2, 0.0f));
}
__device__ __forceinline__ float2 df_sqrt(float2 a) {
  if (!(a.x > 0.0f)) return make_float2(0.0f, 0.0f);
  const float x = sqrtf(a.x);
  const float2 r = df_add(a, df_neg(df_mul(make_float2(x, 0.0f), make_float2(x, 0.0f))));
  return df_add(make_float2(x, 0.0f), make_float2(r.x / (2.0f * x), 0.0f));
}

// Per chart: the dense inverse of its last block (m <= kDirect rows), by a right-looking
// Cholesky factorisation and a right-looking forward substitution of L Y = I, then
// A^-1 = Y^T Y, all in double-float pairs (FP32 FMA pipe; GB300's FP64 pipe made the FP64
// form of this kernel throughput-bound).  Pivot floor: on a nearly singular chart (kappa ~
// 1e10: a long chain pinned at its ends) the smallest eigenvalue of the coarse block is below
// the rounding of its entries; the floor 1e-6 |a_jj| keeps the factor real and leaves that
// one mode to the outer Krylov iteration.  A zero or non-finite pivot sets *bad.
__global__ void __launch_bounds__(kFactorThreads) k_direct_factor(const int32_t* __restrict__ final_lvl,
                                                                  const int64_t* const* __restrict__ lvl_chart_row,
                                                                  const int32_t* const* __restrict__ lvl_rp,
                                                                  const int32_t* const* __restrict__ lvl_cols,
                                                                  const double* const* __restrict__ lvl_vals,
                                                                  const int64_t* __restrict__ fac_off, float* __restrict__ fac,
                                                                  int* __restrict__ bad) {
  extern __shared__ float2 dsm[];
  float2* M = dsm;                      // m x m, row-major: the lower triangle becomes L
  float2* Y = dsm + kDirect * kDirect;  // starts as I; row i becomes (L^-1)[i] at step i
  __shared__ float dg0[kDirect];        // |a_jj| before the factorisation (the pivot floor)
  const int c = blockIdx.x;
  const int f = final_lvl[c];
  if (f < 0) return;
  const int64_t r0 = lvl_chart_row[f][c];
  const int m = (int)(lvl_chart_row[f][c + 1] - r0);
  if (m <= 0 || m > kDirect) return;
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    M[t] = make_float2(0.0f, 0.0f);
    Y[t] = make_float2((t / m) == (t % m) ? 1.0f : 0.0f, 0.0f);
  }
  for (int t = threadIdx.x; t < m; t += blockDim.x) dg0[t] = 0.0f;
  __syncthreads();
  for (int r = threadIdx.x; r < m; r += blockDim.x) {
    const int64_t row = r0 + r;
    for (int e = lvl_rp[f][row]; e < lvl_rp[f][row + 1]; ++e) {
      const int64_t col = lvl_cols[f][e] - r0;
      if (col >= 0 && col < m) {
        const double v = lvl_vals[f][e];
        const float hi = (float)v;
        M[r * m + col] = make_float2(hi, (float)(v - (double)hi));
        if (col == r) dg0[r] = fabsf(hi);
      }
    }
  }
  __syncthreads();
  // L: column j scaled by its pivot, then the trailing block updated (entries in parallel)
  for (int j = 0; j < m; ++j) {
    if (threadIdx.x == 0) {
      float2 d = M[j * m + j];
      const float fl = 1e-6f * dg0[j];
      if (!(d.x > fl)) d = make_float2(fl, 0.0f);
      if (!(d.x > 0.0f) || !isfinite(d.x)) {  // a zero or non-finite diagonal
        atomicExch(bad, 1);
        d = make_float2(1e-30f, 0.0f);
      }
      M[j * m + j] = df_sqrt(d);
    }
    __syncthreads();
    const float2 piv = M[j * m + j];
    for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) M[i * m + j] = df_div(M[i * m + j], piv);
    __syncthreads();
    const int w = m - j - 1;  // trailing block: rows and columns j+1 .. m-1, lower triangle
    for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
      const int i = j + 1 + t / w, k = j + 1 + t % w;
      if (k > i) continue;
      M[i * m + k] = df_add(M[i * m + k], df_neg(df_mul(M[i * m + j], M[k * m + j])));
    }
    __syncthreads();
  }
  // Y = L^-1: row i scaled by L_ii, then the rows below updated
  for (int i = 0; i < m; ++i) {
    const float2 lii = M[i * m + i];
    for (int j = threadIdx.x; j <= i; j += blockDim.x) Y[i * m + j] = df_div(Y[i * m + j], lii);
    __syncthreads();
    const int rows = m - i - 1;
    for (int t = threadIdx.x; t < rows * (i + 1); t += blockDim.x) {
      const int k = i + 1 + t / (i + 1), j = t % (i + 1);
      Y[k * m + j] = df_add(Y[k * m + j], df_neg(df_mul(M[k * m + i], Y[i * m + j])));
    }
    __syncthreads();
  }
  // A^-1 = Y^T Y: (A^-1)[i][k] = sum_{j >= max(i,k)} Y[j][i] Y[j][k], for i <= k and mirrored
  float* Ainv = fac + fac_off[c];
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    const int i = t / m, k = t % m;
    if (i > k) continue;
    float2 s = make_float2(0.0f, 0.0f);
    for (int j = k; j < m; ++j) s = df_add(s, df_mul(Y[j * m + i], Y[j * m + k]));
    Ainv[i * m + k] = s.x;
    Ainv[k * m + i] = s.x;
  }
}

// ---------------------------------------------------------------- apply kernels
template <int NR>
struct F {
  float c[NR];
};
template <int NR>
__device__ __forceinline__ F<NR> ldf(const float* p, int64_t i) {
  F<NR> r;
  if constexpr (NR == 2) {
    float2 t = reinterpret_cast<const float2*>(p)[i];
    r.c[0] = t.x;
    r.c[1] = t.y;
  } else {
    r.c[0] = p[i];
  }
  return r;
}
template <int NR>
__device__ __forceinline__ void stf(float* p, int64_t i, const F<NR>& v) {
  if constexpr (NR == 2) reinterpret_cast<float2*>(p)[i] = make_float2(v.c[0], v.c[1]);
  else p[i] = v.c[0];
}

// The level kernels run over chart-aligned row tiles (one CTA per tile, one chart-state
// check per CTA) as CSR-vector: LPR lanes per row, each lane covering K entries in one
// unrolled sweep (longer rows finish in a remainder loop), U rows in flight per sub-warp,
// block-uniform trip counts (every lane takes part in the shuffles).  One generic row loop,
// four row operations; the shape per operator comes from its mean row length.
struct LvlTiles {
  const int64_t* tab;    // [begin, end) pairs
  const int32_t* chart;  // chart of each tile
  int64_t n;
};

template <int NR>
struct RowIn {
  int lo, hi;
};

// Generic: for each row i of the tile, s = sum_e w(e) * g(col(e)); then fin(i, s).
template <int NR, int LPR, int U, int K, class Col, class W, class G, class Fin>
__device__ __forceinline__ void tile_rows(int64_t beg, int64_t end, const int64_t* ptr64, const int32_t* ptr32, Col cols,
                                          W w, G g, Fin fin) {
  const int sub = threadIdx.x % LPR;
  const int rpp = kAmgThreads / LPR;
  for (int64_t base = beg; base < end; base += (int64_t)rpp * U) {
    int64_t lo[U], hi[U];
    int32_t rb[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      rb[u] = cols.row_base(i);
      const bool valid = i < end;
      lo[u] = valid ? (ptr64 ? ptr64[i] : (int64_t)ptr32[i]) : 0;
      hi[u] = valid ? (ptr64 ? ptr64[i + 1] : (int64_t)ptr32[i + 1]) : 0;
    }
    float av[U][K];
    int cv[U][K];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int64_t e = lo[u] + sub + k * LPR;
        const bool in = e < hi[u];
        av[u][k] = in ? w(e) : 0.0f;
        cv[u][k] = in ? cols(e, rb[u]) : -1;
      }
    F<NR> s[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int c = 0; c < NR; ++c) s[u].c[c] = 0.0f;
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (cv[u][k] >= 0) {
          const F<NR> v = g(cv[u][k]);
#pragma unroll
          for (int c = 0; c < NR; ++c) s[u].c[c] += av[u][k] * v.c[c];
        }
      for (int64_t e = lo[u] + sub + K * LPR; e < hi[u]; e += LPR) {
        const float a = w(e);
        const F<NR> v = g(cols(e, rb[u]));
#pragma unroll
        for (int c = 0; c < NR; ++c) s[u].c[c] += a * v.c[c];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < NR; ++c) s[u].c[c] += __shfl_xor_sync(0xffffffffu, s[u].c[c], o, LPR);
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      if (sub == 0 && i < end) fin(i, s[u]);
    }
  }
}

// tile_rows with the row pointers read through a functor (a staged tile in shared memory).
template <int NR, int LPR, int U, int K, class RP, class Col, class W, class G, class Fin>
__device__ __forceinline__ void tile_rows_rp(int64_t beg, int64_t end, RP rpf, Col cols, W w, G g, Fin fin) {
  const int sub = threadIdx.x % LPR;
  const int rpp = kAmgThreads / LPR;
  for (int64_t base = beg; base < end; base += (int64_t)rpp * U) {
    int64_t lo[U], hi[U];
    int32_t rb[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      rb[u] = cols.row_base(i);
      const bool valid = i < end;
      lo[u] = valid ? rpf(i) : 0;
      hi[u] = valid ? rpf(i + 1) : 0;
    }
    float av[U][K];
    int cv[U][K];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int64_t e = lo[u] + sub + k * LPR;
        const bool in = e < hi[u];
        av[u][k] = in ? w(e) : 0.0f;
        cv[u][k] = in ? cols(e, rb[u]) : -1;
      }
    F<NR> s[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int c = 0; c < NR; ++c) s[u].c[c] = 0.0f;
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (cv[u][k] >= 0) {
          const F<NR> v = g(cv[u][k]);
#pragma unroll
          for (int c = 0; c < NR; ++c) s[u].c[c] += av[u][k] * v.c[c];
        }
      for (int64_t e = lo[u] + sub + K * LPR; e < hi[u]; e += LPR) {
        const float a = w(e);
        const F<NR> v = g(cols(e, rb[u]));
#pragma unroll
        for (int c = 0; c < NR; ++c) s[u].c[c] += a * v.c[c];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < NR; ++c) s[u].c[c] += __shfl_xor_sync(0xffffffffu, s[u].c[c], o, LPR);
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      if (sub == 0 && i < end) fin(i, s[u]);
    }
  }
}

// Down 1: x = w D^-1 b;  t = b - A x  (x of neighbours formed on the fly).
template <int NR, int LPR, int U, int K, int NW>
__global__ void __launch_bounds__(kAmgThreads) k_smooth_down(LvlTiles T, const int32_t* __restrict__ done,
                                                             const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                                             const uint16_t* __restrict__ c16,
                                                             const int32_t* __restrict__ cbase,
                                                             const float* __restrict__ vals, const float* __restrict__ dinv,
                                                             const float* __restrict__ b, float* __restrict__ x,
                                                             float* __restrict__ t) {
  const int64_t tl = blockIdx.x;
  const int32_t ch = T.chart[tl];
  if (done[ch]) return;
  auto run = [&](auto colf) {
  tile_rows<NR, LPR, U, K>(
      T.tab[2 * tl], T.tab[2 * tl + 1], nullptr, rp, colf, [&](int64_t e) { return vals[e]; },
      [&](int32_t j) {
        F<NR> v = ldf<NR>(b, j);
        const float wd = kOmega * dinv[j];
#pragma unroll
        for (int c = 0; c < NR; ++c) v.c[c] *= wd;
        return v;
      },
      [&](int64_t i, const F<NR>& s) {
        const F<NR> bi = ldf<NR>(b, i);
        F<NR> xi, ti;
        const float wd = kOmega * dinv[i];
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          xi.c[c] = wd * bi.c[c];
          ti.c[c] = bi.c[c] - s.c[c];
        }
        if (x) stf<NR>(x, i, xi);  // (the tentative-P cycle forms it again on the way up)
        stf<NR>(t, i, ti);
      });
  };
  if constexpr (NW == 1) run(ColsNarrow{c16, cbase[ch]});
  else if constexpr (NW == 2) run(ColsRowRel{c16});
  else run(ColsWide{cols});
}

// Staged forms of the level-0 smoothers: each CTA first stages its tile's row pointers, FP32
// values and column stream into shared memory by bulk asynchronous copies (stage_rows, a
// bounded wait that sets *err) and then runs the same row loop from there; the same
// arithmetic in the same order, so the same results.
template <class ColsT, int NW>
struct StagedOp {
  StagedRows S;
  int32_t cb;
  __device__ __forceinline__ int64_t rp(int64_t i) const { return (int64_t)S.rp[i - S.fr]; }
  __device__ __forceinline__ float w(int64_t e) const { return reinterpret_cast<const float*>(S.v)[e - S.fv]; }
  __device__ __forceinline__ int32_t row_base(int64_t i) const { return narrow_row_base<NW>(cb, i); }
  __device__ __forceinline__ int32_t operator()(int64_t e, int32_t rb) const {
    if constexpr (NW != 0) return rb + (int32_t)(reinterpret_cast<const uint16_t*>(S.c)[e - S.fc]);
    else return reinterpret_cast<const int32_t*>(S.c)[e - S.fc];
  }
};

template <int NR, int LPR, int U, int K, int NW>
__global__ void __launch_bounds__(kAmgThreads) k_smooth_down_st(LvlTiles T, const int32_t* __restrict__ done,
                                                                const int32_t* __restrict__ rp,
                                                                const int32_t* __restrict__ cols,
                                                                const uint16_t* __restrict__ c16,
                                                                const int32_t* __restrict__ cbase,
                                                                const float* __restrict__ vals,
                                                                const float* __restrict__ dinv,
                                                                const float* __restrict__ b, float* __restrict__ x,
                                                                float* __restrict__ t, int64_t limit, int* err) {
  extern __shared__ __align__(16) unsigned char stage[];
  const int64_t tl = blockIdx.x;
  const int32_t ch = T.chart[tl];
  if (done[ch]) return;
  const int64_t beg = T.tab[2 * tl], end = T.tab[2 * tl + 1];
  StagedOp<int, NW> op;
  if (!stage_rows(stage, rp, beg, end, vals, 4, NW ? (const void*)c16 : (const void*)cols, NW ? 2 : 4, limit,
                  err, op.S))
    return;
  op.cb = NW == 1 ? cbase[ch] : 0;
  tile_rows_rp<NR, LPR, U, K>(
      beg, end, [&](int64_t i) { return op.rp(i); }, op,
      [&](int64_t e) { return op.w(e); },
      [&](int32_t j) {
        F<NR> v = ldf<NR>(b, j);
        const float wd = kOmega * dinv[j];
#pragma unroll
        for (int c = 0; c < NR; ++c) v.c[c] *= wd;
        return v;
      },
      [&](int64_t i, const F<NR>& sv) {
        const F<NR> bi = ldf<NR>(b, i);
        F<NR> xi, ti;
        const float wd = kOmega * dinv[i];
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          xi.c[c] = wd * bi.c[c];
          ti.c[c] = bi.c[c] - sv.c[c];
        }
        if (x) stf<NR>(x, i, xi);
        stf<NR>(t, i, ti);
      });
}

template <int NR, int LPR, int U, int K, int NW>
__global__ void __launch_bounds__(kAmgThreads) k_smooth_up_st(LvlTiles T, const int32_t* __restrict__ done,
                                                              const int32_t* __restrict__ rp,
                                                              const int32_t* __restrict__ cols,
                                                              const uint16_t* __restrict__ c16,
                                                              const int32_t* __restrict__ cbase,
                                                              const float* __restrict__ vals,
                                                              const float* __restrict__ dinv,
                                                              const float* __restrict__ b, const float* __restrict__ y,
                                                              float* __restrict__ x, int64_t limit, int* err) {
  extern __shared__ __align__(16) unsigned char stage[];
  const int64_t tl = blockIdx.x;
  const int32_t ch = T.chart[tl];
  if (done[ch]) return;
  const int64_t beg = T.tab[2 * tl], end = T.tab[2 * tl + 1];
  StagedOp<int, NW> op;
  if (!stage_rows(stage, rp, beg, end, vals, 4, NW ? (const void*)c16 : (const void*)cols, NW ? 2 : 4, limit,
                  err, op.S))
    return;
  op.cb = NW == 1 ? cbase[ch] : 0;
  tile_rows_rp<NR, LPR, U, K>(
      beg, end, [&](int64_t i) { return op.rp(i); }, op,
      [&](int64_t e) { return op.w(e); }, [&](int32_t j) { return ldf<NR>(y, j); },
      [&](int64_t i, const F<NR>& sv) {
        const F<NR> bi = ldf<NR>(b, i), yi = ldf<NR>(y, i);
        F<NR> xi;
        const float wd = kOmega * dinv[i];
#pragma unroll
        for (int c = 0; c < NR; ++c) xi.c[c] = yi.c[c] + wd * (bi.c[c] - sv.c[c]);
        stf<NR>(x, i, xi);
      });
}

// the largest tile's nonzeros and rows of a level operator
__global__ void k_lvl_tile_max(LvlTiles T, const int32_t* __restrict__ rp, unsigned long long* __restrict__ mx) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.n) return;
  const int64_t b = T.tab[2 * t], e = T.tab[2 * t + 1];
  atomicMax(mx, (unsigned long long)(rp[e] - rp[b]));
  atomicMax(mx + 1, (unsigned long long)(e - b));
}

// Restrict: b_c = R t over the coarse rows (tiles of the coarse level).
template <int NR, int LPR, int U, int K>
__global__ void __launch_bounds__(kAmgThreads) k_restrict(LvlTiles T, const int32_t* __restrict__ done,
                                                          const int64_t* __restrict__ roff, const int32_t* __restrict__ rc,
                                                          const float* __restrict__ rv, const float* __restrict__ t,
                                                          float* __restrict__ bc) {
  const int64_t tl = blockIdx.x;
  if (done[T.chart[tl]]) return;
  tile_rows<NR, LPR, U, K>(
      T.tab[2 * tl], T.tab[2 * tl + 1], roff, nullptr, ColsWide{rc}, [&](int64_t e) { return rv[e]; },
      [&](int32_t j) { return ldf<NR>(t, j); }, [&](int64_t I, const F<NR>& s) { stf<NR>(bc, I, s); });
}

// Up 1: y = x + alpha_c P x_c (alpha_c = 1: plain; > 1: over-correction of an unsmoothed
// (piecewise-constant) coarse space, which underestimates the smooth error).
template <int NR, int LPR, int U, int K>
__global__ void __launch_bounds__(kAmgThreads) k_prolong_add(LvlTiles T, const int32_t* __restrict__ done,
                                                             const int64_t* __restrict__ poff, const int32_t* __restrict__ pc,
                                                             const float* __restrict__ pv, const float* __restrict__ xc,
                                                             const float* __restrict__ x, float* __restrict__ y, float alpha_c) {
  const int64_t tl = blockIdx.x;
  if (done[T.chart[tl]]) return;
  tile_rows<NR, LPR, U, K>(
      T.tab[2 * tl], T.tab[2 * tl + 1], poff, nullptr, ColsWide{pc}, [&](int64_t e) { return alpha_c * pv[e]; },
      [&](int32_t j) { return ldf<NR>(xc, j); },
      [&](int64_t i, const F<NR>& s) {
        F<NR> xi;
        if (x) {
          xi = ldf<NR>(x, i);
        } else {
#pragma unroll
          for (int c = 0; c < NR; ++c) xi.c[c] = 0.0f;
        }
#pragma unroll
        for (int c = 0; c < NR; ++c) xi.c[c] += s.c[c];
        stf<NR>(y, i, xi);
      });
}

// K-cycle coarse correction (the K-form of gpu/src/amg.rs:468-639): w = A y over the rows of
// the level's continuing charts, with per-tile partial sums y.t and y.w (FP32 per row, FP64
// per tile, fixed combine order) for the steplength beta = (y.t) / (y.A y), the step along y
// that minimises the A-norm of the error (the K-cycle's published form, Notay and
// Vassilevski).  The reference divides t.t by t.A y instead; with the FP32 cycle that
// quotient is not energy-decreasing, and the outer flexible CG stalled with it (16384
// iterations without converging on charts the V-cycle solves in a few dozen).
template <int NR, int LPR, int U, int K, int NW>
__global__ void __launch_bounds__(kAmgThreads) k_kspmv(LvlTiles T, const int32_t* __restrict__ done,
                                                       const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                                       const uint16_t* __restrict__ c16, const int32_t* __restrict__ cbase,
                                                       const float* __restrict__ vals, const float* __restrict__ y,
                                                       const float* __restrict__ t, float* __restrict__ w,
                                                       double* __restrict__ part) {
  __shared__ double sh[2 * 32];
  const int64_t tl = blockIdx.x;
  const int32_t ch = T.chart[tl];
  if (done[ch]) return;
  double acc[2] = {0.0, 0.0};
  auto run = [&](auto colf) {
    tile_rows<NR, LPR, U, K>(
        T.tab[2 * tl], T.tab[2 * tl + 1], nullptr, rp, colf, [&](int64_t e) { return vals[e]; },
        [&](int32_t j) { return ldf<NR>(y, j); },
        [&](int64_t i, const F<NR>& sv) {
          stf<NR>(w, i, sv);
          const F<NR> ti = ldf<NR>(t, i), yi = ldf<NR>(y, i);
          float yt = 0.0f, yw = 0.0f;
#pragma unroll
          for (int c = 0; c < NR; ++c) {
            yt += yi.c[c] * ti.c[c];
            yw += yi.c[c] * sv.c[c];
          }
          acc[0] += (double)yt;
          acc[1] += (double)yw;
        });
  };
  if constexpr (NW == 1) run(ColsNarrow{c16, cbase[ch]});
  else if constexpr (NW == 2) run(ColsRowRel{c16});
  else run(ColsWide{cols});
  block_sum<2>(acc, sh);
  if (threadIdx.x == 0) {
    part[2 * tl] = acc[0];
    part[2 * tl + 1] = acc[1];
  }
}

// beta per chart from its tiles' partial sums (one CTA per chart, fixed combine order); a
// non-positive or tiny y.A y skips the correction (beta = 0), as the reference guards its
// denominator.
__global__ void __launch_bounds__(128) k_kbeta(const int32_t* __restrict__ done, const int64_t* __restrict__ chart_tile,
                                               const double* __restrict__ part, float* __restrict__ beta) {
  __shared__ double sh[2 * 32];
  const int64_t c = blockIdx.x;
  if (done[c]) return;
  double acc[2] = {0.0, 0.0};
  for (int64_t t = chart_tile[c] + threadIdx.x; t < chart_tile[c + 1]; t += blockDim.x) {
    acc[0] += part[2 * t];
    acc[1] += part[2 * t + 1];
  }
  block_sum<2>(acc, sh);
  if (threadIdx.x == 0) beta[c] = acc[1] > 1e-300 ? (float)(acc[0] / acc[1]) : 0.0f;
}

// x += beta y; t -= beta w (t may be null: the last correction of the level).
template <int NR>
__global__ void __launch_bounds__(kAmgThreads) k_kupdate(LvlTiles T, const int32_t* __restrict__ done,
                                                         const float* __restrict__ beta, const float* __restrict__ y,
                                                         const float* __restrict__ w, float* __restrict__ x,
                                                         float* __restrict__ t) {
  const int64_t tl = blockIdx.x;
  const int32_t ch = T.chart[tl];
  if (done[ch]) return;
  const float b = beta[ch];
  for (int64_t i = T.tab[2 * tl] + threadIdx.x; i < T.tab[2 * tl + 1]; i += blockDim.x) {
    F<NR> xi = ldf<NR>(x, i);
    const F<NR> yi = ldf<NR>(y, i);
#pragma unroll
    for (int c = 0; c < NR; ++c) xi.c[c] += b * yi.c[c];
    stf<NR>(x, i, xi);
    if (t) {
      F<NR> ti = ldf<NR>(t, i);
      const F<NR> wi = ldf<NR>(w, i);
#pragma unroll
      for (int c = 0; c < NR; ++c) ti.c[c] -= b * wi.c[c];
      stf<NR>(t, i, ti);
    }
  }
}

// Up 2: x = y + w D^-1 (b - A y).
template <int NR, int LPR, int U, int K, int NW>
__global__ void __launch_bounds__(kAmgThreads) k_smooth_up(LvlTiles T, const int32_t* __restrict__ done,
                                                           const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                                           const uint16_t* __restrict__ c16,
                                                           const int32_t* __restrict__ cbase,
                                                           const float* __restrict__ vals, const float* __restrict__ dinv,
                                                           const float* __restrict__ b, const float* __restrict__ y,
                                                           float* __restrict__ x) {
  const int64_t tl = blockIdx.x;
  const int32_t ch = T.chart[tl];
  if (done[ch]) return;
  auto run = [&](auto colf) {
  tile_rows<NR, LPR, U, K>(
      T.tab[2 * tl], T.tab[2 * tl + 1], nullptr, rp, colf, [&](int64_t e) { return vals[e]; },
      [&](int32_t j) { return ldf<NR>(y, j); },
      [&](int64_t i, const F<NR>& s) {
        const F<NR> bi = ldf<NR>(b, i), yi = ldf<NR>(y, i);
        F<NR> xi;
        const float wd = kOmega * dinv[i];
#pragma unroll
        for (int c = 0; c < NR; ++c) xi.c[c] = yi.c[c] + wd * (bi.c[c] - s.c[c]);
        stf<NR>(x, i, xi);
      });
  };
  if constexpr (NW == 1) run(ColsNarrow{c16, cbase[ch]});
  else if constexpr (NW == 2) run(ColsRowRel{c16});
  else run(ColsWide{cols});
}

// Up, tentative prolongator (one 1 per row at agg[i]): the prolongation and the
// post-smoothing in one pass, x = y + w D^-1 (b - A y) with y_j = w D^-1_j b_j +
// alpha_c x_c[agg[j]] formed on the fly for every neighbour (the pre-smoothed x is not
// stored and y is never written).
template <int NR, int LPR, int U, int K, int NW>
__global__ void __launch_bounds__(kAmgThreads) k_smooth_up_t(LvlTiles T, const int32_t* __restrict__ done,
                                                             const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                                             const uint16_t* __restrict__ c16,
                                                             const int32_t* __restrict__ cbase,
                                                             const float* __restrict__ vals, const float* __restrict__ dinv,
                                                             const float* __restrict__ b, const int32_t* __restrict__ agg,
                                                             const float* __restrict__ xc, float alpha_c,
                                                             float* __restrict__ x) {
  const int64_t tl = blockIdx.x;
  const int32_t ch = T.chart[tl];
  if (done[ch]) return;
  auto yval = [&](int64_t j) {
    F<NR> v = ldf<NR>(b, j);
    const float wd = kOmega * dinv[j];
    const F<NR> c = ldf<NR>(xc, agg[j]);
#pragma unroll
    for (int k = 0; k < NR; ++k) v.c[k] = wd * v.c[k] + alpha_c * c.c[k];
    return v;
  };
  auto run = [&](auto colf) {
  tile_rows<NR, LPR, U, K>(
      T.tab[2 * tl], T.tab[2 * tl + 1], nullptr, rp, colf, [&](int64_t e) { return vals[e]; },
      [&](int32_t j) { return yval(j); },
      [&](int64_t i, const F<NR>& s) {
        const F<NR> bi = ldf<NR>(b, i), yi = yval(i);
        F<NR> xi;
        const float wd = kOmega * dinv[i];
#pragma unroll
        for (int c = 0; c < NR; ++c) xi.c[c] = yi.c[c] + wd * (bi.c[c] - s.c[c]);
        stf<NR>(x, i, xi);
      });
  };
  if constexpr (NW == 1) run(ColsNarrow{c16, cbase[ch]});
  else if constexpr (NW == 2) run(ColsRowRel{c16});
  else run(ColsWide{cols});
}

// Direct solve of every chart at its last level: x = A^-1 b with the dense inverse (one CTA
// of kDirect threads per chart, thread i forms row i; A^-1 is symmetric, so row i is read as
// column i and the loads coalesce across threads).
template <int NR>
__global__ void __launch_bounds__(kDirect) k_direct_solve(const int32_t* __restrict__ final_lvl, const int32_t* __restrict__ done,
                                                          const int64_t* const* __restrict__ lvl_chart_row,
                                                          float* const* __restrict__ lvl_b, float* const* __restrict__ lvl_x,
                                                          const float* const* __restrict__ lvl_dinv,
                                                          const int64_t* __restrict__ fac_off, const float* __restrict__ fac,
                                                          int lo, int hi) {
  __shared__ float bs[NR][kDirect];
  const int c = blockIdx.x;
  const int f = final_lvl[c];
  if (f < lo || f > hi || done[c]) return;  // only charts whose last level is in [lo, hi]
  const int64_t r0 = lvl_chart_row[f][c];
  const int m = (int)(lvl_chart_row[f][c + 1] - r0);
  if (m <= 0) return;
  const float* b = lvl_b[f];
  float* x = lvl_x[f];
  const int i = threadIdx.x;
  if (m > kDirect) {  // aggregation stalled above the dense limit: x = D^-1 b
    const float* dv = lvl_dinv[f];
    for (int r = i; r < m; r += blockDim.x)
#pragma unroll
      for (int k = 0; k < NR; ++k) x[NR * (r0 + r) + k] = dv[r0 + r] * b[NR * (r0 + r) + k];
    return;
  }
  if (i < m)
#pragma unroll
    for (int k = 0; k < NR; ++k) bs[k][i] = b[NR * (r0 + i) + k];
  __syncthreads();
  if (i >= m) return;
  const float* Ainv = fac + fac_off[c];
  float s[NR];
#pragma unroll
  for (int k = 0; k < NR; ++k) s[k] = 0.0f;
  for (int j = 0; j < m; ++j) {
    const float a = Ainv[j * m + i];
#pragma unroll
    for (int k = 0; k < NR; ++k) s[k] += a * bs[k][j];
  }
#pragma unroll
  for (int k = 0; k < NR; ++k) x[NR * (r0 + i) + k] = s[k];
}

}  // namespace

// ---------------------------------------------------------------- host side
struct AmgLevelDev {
  int64_t n = 0, nnz = 0, n_next = 0, n_pnnz = 0;
  std::vector<int64_t> h_chart_row;
  int64_t* chart_row = nullptr;
  int32_t* row_chart = nullptr;
  int32_t *rp = nullptr, *cols = nullptr;
  float *vals = nullptr, *dinv = nullptr;
  double* vals64 = nullptr;  // the operator in FP64 (the coarsest level's dense factors)
  float* vals_lo = nullptr;  // (vals, vals_lo): the operator as double-float pairs (the Galerkin products' input)
  float2* vdf = nullptr;     // a coarse level's pairs as its Galerkin product wrote them
  // transfer to the next level (rows of charts that continue below this level)
  int64_t* poff = nullptr;
  int32_t* pc = nullptr;
  float* pv = nullptr;
  int64_t* roff = nullptr;
  int32_t* rc = nullptr;
  float* rv = nullptr;
  float *b = nullptr, *x = nullptr, *y = nullptr, *t = nullptr;
  int32_t* agg = nullptr;  // aggregate of each row (the tentative prolongator), -1 if none
  bool smoothed = false;   // transfer to the next level by a smoothed prolongator (else tentative)
  const uint16_t* c16 = nullptr;  // 16-bit column stream (see ColsNarrow, ColsRowRel)
  bool rowrel = false;            // c16 holds row-relative offsets
  const int32_t* cbase = nullptr;
  LvlTiles cont{nullptr, nullptr, 0};  // tiles over rows whose chart continues below this level
  LvlTiles all{nullptr, nullptr, 0};   // tiles over every row of this level
  // K-cycle levels: chart c's continuing tiles are [cont_chart_tile[c], cont_chart_tile[c + 1]);
  // w = A y, the tiles' partial sums and the per-chart steplength
  const int64_t* cont_chart_tile = nullptr;
  float* w = nullptr;
  double* kpart = nullptr;
  float* kbeta = nullptr;
  size_t stage_smem = 0;  // > 0: the smoothers stage their tiles (bytes of shared memory)
};

struct AmgHierarchy {
  int nrhs = 2;
  bool smoothed = false;  // smoothed prolongators (AMG-SA) on the first sa_levels levels; else tentative
  int sa_levels = 0;
  int64_t n_charts = 0;
  std::vector<AmgLevelDev> lv;
  int32_t* final_lvl = nullptr;
  int64_t* fac_off = nullptr;
  float* fac = nullptr;
  const int64_t** d_lvl_chart_row = nullptr;
  float** d_lvl_b = nullptr;
  float** d_lvl_x = nullptr;
  const float** d_lvl_dinv = nullptr;
  std::vector<int32_t> h_final;
  int64_t total_rows = 0, total_nnz = 0;
  float alpha_c = 1.0f;
  int k_levels = 0;  // top levels applied in the K-form (two coarse corrections with steplengths)
  int* err = nullptr;  // a staged tile's bounded wait ran out
  int64_t spin_limit = 0;
};

namespace {

int64_t read_i64(Ctx& ctx, const int64_t* d) {
  int64_t* h = static_cast<int64_t*>(ctx.pinned.get(sizeof(int64_t)));
  RUV_CUDA(cudaMemcpyAsync(h, d, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx.stream));
  RUV_CUDA(cudaStreamSynchronize(ctx.stream));
  return *h;
}

// Two-pass row build from a count kernel: counts -> offsets (int64, n + 1) and the total.
int64_t offsets_from_counts(Ctx& ctx, const int32_t* cnt, int64_t n, int64_t* off, const std::string& tag) {
  exclusive_scan(cnt, off, n, ctx.ws, ctx.stream, tag);
  return read_i64(ctx, off + n);
}

// Work areas of the sparse products: the staging rows and their counts, and the rows listed
// for the large-table kernel (count at list_n on the device, h1 on the host).
struct GalWork {
  int32_t* list = nullptr;
  int32_t* list_n = nullptr;
  int* ovf = nullptr;
  int32_t* sn = nullptr;
  int32_t* st_key = nullptr;
  float2* st_val = nullptr;
  float* st_dinv = nullptr;
  int hs = 0;     // staged entries per row
  int lanes = 0;  // lanes per row of the first pass
  int32_t h1 = 0;
  bool debug = false;
  std::chrono::steady_clock::time_point t0;
};
constexpr int kGalWarps = 8;
constexpr int kGalBigH = 8192;  // large table: 4096 distinct keys, 128 KB of shared memory

template <int MODE, int G, int H, int WARPS, bool DIAG, class OP, class OL, class IP, class IL, class KeyF>
void launch_gal(cudaStream_t s, int64_t nrows, const int32_t* list, const uint8_t* active, const OP* o_ptr,
                const int32_t* o_idx, OL o_val, const IP* i_ptr, const int32_t* i_idx, IL i_val, KeyF keyf,
                const GalOut& out) {
  constexpr int SUB = 32 / G;
  constexpr size_t smem = GalSmem<G, H>::bytes * WARPS * SUB;
  auto k = k_gal_hash<MODE, G, H, WARPS, DIAG, OP, OL, IP, IL, KeyF>;
  if (smem > 48 * 1024) RUV_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k<<<div_up(nrows, (int64_t)WARPS * SUB), 32 * WARPS, smem, s>>>(nrows, list, active, o_ptr, o_idx, o_val, i_ptr, i_idx,
                                                                 i_val, keyf, out);
  count_launches(1);
  RUV_LAUNCH_CHECK();
}

inline double env_or(const char* name, double dflt) {
  const char* e = std::getenv(name);
  return e ? std::atof(e) : dflt;
}

// First half of a sparse product over `nrows` rows (`avg`: the mean products per row, which
// picks 8, 16 or 32 lanes per row with tables of 64, 128 or 256 slots -- more rows in flight
// for short rows).  Every row is evaluated once into the staging area; rows with more distinct
// keys than the table holds are counted by the large-table kernel.  cnt holds every row's
// count on return.
template <bool DIAG, class OP, class OL, class IP, class IL, class KeyF>
void gal_count(Ctx& ctx, GalWork& g, int64_t nrows, double avg, const uint8_t* active, const OP* o_ptr,
               const int32_t* o_idx, OL o_val, const IP* i_ptr, const int32_t* i_idx, IL i_val, KeyF keyf,
               int32_t* cnt) {
  cudaStream_t s = ctx.stream;
  g.h1 = 0;
  if (nrows <= 0) return;
  if (g.debug) {
    RUV_CUDA(cudaStreamSynchronize(s));
    g.t0 = std::chrono::steady_clock::now();
  }
  const double t8 = env_or("RUV_GAL_T8", 32.0), t16 = env_or("RUV_GAL_T16", 48.0);
  g.lanes = avg < t8 ? 8 : avg < t16 ? 16 : 32;
  g.hs = g.lanes == 8 ? GalSmem<8, 64>::HS : g.lanes == 16 ? GalSmem<16, 128>::HS : GalSmem<32, 256>::HS;
  g.sn = ctx.ws.get<int32_t>("amg.gal_sn", nrows);
  g.st_key = ctx.ws.get<int32_t>("amg.gal_key", nrows * g.hs);
  g.st_val = ctx.ws.get<float2>("amg.gal_val", nrows * g.hs);
  g.st_dinv = DIAG ? ctx.ws.get<float>("amg.gal_dinv", nrows) : nullptr;
  RUV_CUDA(cudaMemsetAsync(g.list_n, 0, sizeof(int32_t), s));
  GalOut out{cnt, g.sn, g.st_key, g.st_val, nullptr, nullptr, nullptr, g.st_dinv, g.list, g.list_n, g.ovf};
  if (g.lanes == 8)
    launch_gal<2, 8, 64, kGalWarps, DIAG>(s, nrows, nullptr, active, o_ptr, o_idx, o_val, i_ptr, i_idx, i_val, keyf, out);
  else if (g.lanes == 16)
    launch_gal<2, 16, 128, kGalWarps, DIAG>(s, nrows, nullptr, active, o_ptr, o_idx, o_val, i_ptr, i_idx, i_val, keyf, out);
  else
    launch_gal<2, 32, 256, kGalWarps, DIAG>(s, nrows, nullptr, active, o_ptr, o_idx, o_val, i_ptr, i_idx, i_val, keyf, out);
  RUV_CUDA(cudaMemcpyAsync(&g.h1, g.list_n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  if (g.h1 > 0) {
    GalOut o0{cnt, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, g.ovf};
    launch_gal<0, 32, kGalBigH, 1, DIAG>(s, g.h1, g.list, nullptr, o_ptr, o_idx, o_val, i_ptr, i_idx, i_val, keyf, o0);
  }
}

// Second half: staged rows copied to their offsets, listed rows evaluated again by the
// large-table kernel straight into place.
template <bool DIAG, class OP, class OL, class IP, class IL, class KeyF>
void gal_fill(Ctx& ctx, GalWork& g, int64_t nrows, const OP* o_ptr, const int32_t* o_idx, OL o_val,
              const IP* i_ptr, const int32_t* i_idx, IL i_val, KeyF keyf, const int64_t* off, int32_t* oc,
              float2* ov, float* adinv) {
  cudaStream_t s = ctx.stream;
  if (nrows <= 0) return;
  k_gal_copy<<<div_up(nrows * 8, 256), 256, 0, s>>>(nrows, g.hs, g.sn, g.st_key, g.st_val, off, oc, ov);
  count_launches(1);
  if (DIAG) {
    RUV_CUDA(cudaMemcpyAsync(adinv, g.st_dinv, sizeof(float) * nrows, cudaMemcpyDeviceToDevice, s));
  }
  RUV_LAUNCH_CHECK();
  if (g.h1 > 0) {
    GalOut o1{nullptr, nullptr, nullptr, nullptr, off, oc, ov, adinv, nullptr, nullptr, g.ovf};
    launch_gal<1, 32, kGalBigH, 1, DIAG>(s, g.h1, g.list, nullptr, o_ptr, o_idx, o_val, i_ptr, i_idx, i_val, keyf, o1);
  }
  if (g.debug) {
    RUV_CUDA(cudaStreamSynchronize(s));
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - g.t0).count();
    std::fprintf(stderr, "  product rows %lld: %d lanes per row, large-table rows %d, %.3f ms\n", (long long)nrows,
                 g.lanes, g.h1, ms);
  }
}

}  // namespace

constexpr size_t kStageMaxSmem = 100 * 1024;

template <int NR, int NW>
void stage_attributes_nw() {
#define A(X, UU, KK)                                                                                            \
  RUV_CUDA(cudaFuncSetAttribute(k_smooth_down_st<NR, X, UU, KK, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                (int)kStageMaxSmem));                                                            \
  RUV_CUDA(cudaFuncSetAttribute(k_smooth_up_st<NR, X, UU, KK, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                (int)kStageMaxSmem));
  A(1, 4, 2) A(1, 2, 8) A(2, 2, 4) A(2, 2, 8) A(4, 2, 4) A(8, 2, 4) A(16, 1, 4)
#undef A
}

// Level 0's smoothers stage their tiles into shared memory when RUV_AMG_STAGE=1 and the
// largest tile fits in kStageMaxSmem.
void stage_setup(Ctx& ctx, AmgHierarchy* H) {
  const char* e = std::getenv("RUV_AMG_STAGE");
  if (!(e && e[0] == '1') || H->lv.empty()) return;
  AmgLevelDev& L = H->lv[0];
  if (L.cont.n == 0) return;
  cudaStream_t s = ctx.stream;
  unsigned long long* mx = ctx.ws.get<unsigned long long>("amg.stmax", 2);
  RUV_CUDA(cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), s));
  k_lvl_tile_max<<<div_up(L.cont.n, 256), 256, 0, s>>>(L.cont, L.rp, mx);
  count_launches(1);
  unsigned long long h[2] = {0, 0};
  RUV_CUDA(cudaMemcpyAsync(h, mx, sizeof(h), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  const size_t bytes = stage_bytes((int64_t)h[1], (int64_t)h[0], 4, L.c16 ? 2 : 4);
  if (bytes > kStageMaxSmem) return;
  if (H->nrhs == 2) {
    stage_attributes_nw<2, 0>();
    stage_attributes_nw<2, 1>();
    stage_attributes_nw<2, 2>();
  } else {
    stage_attributes_nw<1, 0>();
    stage_attributes_nw<1, 1>();
    stage_attributes_nw<1, 2>();
  }
  H->err = ctx.ws.get<int>("amg.err", 1);
  RUV_CUDA(cudaMemsetAsync(H->err, 0, sizeof(int), s));
  const char* le = std::getenv("RUV_SPIN_LIMIT");
  H->spin_limit = le ? std::max<int64_t>(1, std::atoll(le)) : (int64_t(1) << 22);
  L.stage_smem = bytes;
}

AmgHierarchy* amg_setup(Ctx& ctx, const DevSystem& sys, bool smooth, std::string& info) {
  cudaStream_t s = ctx.stream;
  const int B = kAmgThreads;
  const int64_t NC = sys.n_charts;
  std::unique_ptr<AmgHierarchy> H(new AmgHierarchy());
  H->nrhs = sys.nrhs;
  H->smoothed = smooth;
  H->n_charts = NC;
  // smoothed prolongators on the first sa_levels levels, tentative below (the coarse levels of a
  // smoothed hierarchy are the densest: their products and cycles cost the most)
  H->sa_levels = smooth ? kSaLevels : 0;
  if (const char* e = std::getenv("RUV_AMG_SA_LEVELS")) H->sa_levels = smooth ? std::max(0, std::atoi(e)) : 0;
  H->alpha_c = 1.5f;  // over-correct the piecewise-constant coarse space of tentative levels
  if (const char* e = std::getenv("RUV_AMG_ALPHA")) H->alpha_c = (float)std::atof(e);
  if (const char* e = std::getenv("RUV_AMG_KCYCLE")) H->k_levels = std::max(0, std::atoi(e));
  float strong = kStrong;  // matching candidates: couplings >= strong * the row's strongest
  if (const char* e = std::getenv("RUV_AMG_STRONG")) strong = (float)std::atof(e);
  int pmax = kPMaxRow;
  if (const char* e = std::getenv("RUV_AMG_PMAX")) pmax = std::max(1, std::min(kAccCap, std::atoi(e)));
  int rounds = kPairRounds;  // proposal rounds of each matching pass
  if (const char* e = std::getenv("RUV_AMG_ROUNDS")) rounds = std::max(1, std::atoi(e));
  // group matching over a group graph built once per level (RUV_AMG_GROUP_GRAPH=0: strengths
  // accumulated again in every round; the same aggregates)
  const char* gg_env = std::getenv("RUV_AMG_GROUP_GRAPH");
  const bool graph = !(gg_env && gg_env[0] == '0');
  cudaEvent_t t_setup0;
  RUV_CUDA(cudaEventCreate(&t_setup0));
  RUV_CUDA(cudaEventRecord(t_setup0, s));
  int* ovf = ctx.ws.get<int>("amg.overflow", 8);
  RUV_CUDA(cudaMemsetAsync(ovf, 0, 8 * sizeof(int), s));
  const bool debug = std::getenv("RUV_AMG_DEBUG") != nullptr;
  const char* narrow_env = std::getenv("RUV_NARROW_COLS");
  const bool narrow = !(narrow_env && narrow_env[0] == '0');
  {
    AmgLevelDev L0;
    L0.n = sys.n_rows;
    L0.nnz = sys.nnz;
    L0.h_chart_row = sys.h_chart_row;
    L0.chart_row = sys.chart_row;
    L0.rp = sys.row_ptr;
    L0.cols = sys.cols;
    L0.vals = sys.vals32;
    L0.vals64 = sys.vals;
    L0.vals_lo = sys.vals_lo;
    if (!L0.vals_lo && L0.nnz > 0) {  // (the assembly formed no split: form it here)
      L0.vals_lo = ctx.ws.get<float>("amg.l0.lo", L0.nnz);
      k_lo_half<<<div_up(L0.nnz, B), B, 0, s>>>(L0.nnz, sys.vals, sys.vals32, L0.vals_lo);
      count_launches(1);
    }
    L0.c16 = sys.cols16;
    L0.cbase = sys.cbase;
    L0.rowrel = sys.rowrel16;
    L0.dinv = ctx.ws.get<float>("amg.l0.dinv", L0.n);
    if (L0.n > 0) {
      k_f64_f32_inv<<<div_up(L0.n, B), B, 0, s>>>(L0.n, sys.diag, L0.dinv);
      count_launches(1);
    }
    H->lv.push_back(L0);
  }
  H->h_final.assign(NC, -1);
  std::vector<int32_t> cont(NC, 0);
  for (int lvl = 0; lvl < kMaxLevels; ++lvl) {
    const bool sm = lvl < H->sa_levels;  // this level's prolongator is smoothed
    const std::string tag = "amg.l" + std::to_string(lvl);
    AmgLevelDev& L = H->lv[lvl];
    int64_t n_cont = 0;
    for (int64_t c = 0; c < NC; ++c) {
      if (H->h_final[c] >= 0) {
        cont[c] = 0;
        continue;
      }
      const int64_t m = L.h_chart_row[c + 1] - L.h_chart_row[c];
      bool stalled = false;
      if (lvl > 0) {
        const AmgLevelDev& P = H->lv[lvl - 1];
        const int64_t mf = P.h_chart_row[c + 1] - P.h_chart_row[c];
        stalled = (double)m > 0.85 * (double)mf;
      }
      if (m <= kDirect || lvl == kMaxLevels - 1 || stalled) {
        H->h_final[c] = lvl;
        cont[c] = 0;
      } else {
        cont[c] = 1;
        ++n_cont;
      }
    }
    int32_t* d_cont = ctx.ws.get<int32_t>(tag + ".cont", NC);
    RUV_CUDA(cudaMemcpyAsync(d_cont, cont.data(), sizeof(int32_t) * NC, cudaMemcpyHostToDevice, s));
    L.row_chart = ctx.ws.get<int32_t>(tag + ".row_chart", L.n);
    uint8_t* active = ctx.ws.get<uint8_t>(tag + ".active", L.n);
    if (L.n > 0) {
      k_row_chart<<<div_up(L.n, B), B, 0, s>>>(L.n, L.chart_row, NC, d_cont, L.row_chart, active);
      count_launches(1);
    }
    RUV_CUDA(cudaStreamSynchronize(s));  // `cont` is reused by the next level
    if (n_cont == 0) break;
    // ---- aggregation: pairs of rows, then pairs of pairs
    int32_t* mate = ctx.ws.get<int32_t>(tag + ".mate", L.n);
    int32_t* prop = ctx.ws.get<int32_t>(tag + ".prop", L.n);
    RUV_CUDA(cudaMemsetAsync(mate, 0xff, sizeof(int32_t) * L.n, s));
    for (int r = 0; r < rounds; ++r) {
      k_propose<<<div_up(L.n, B), B, 0, s>>>(L.n, L.rp, L.cols, L.vals, active, mate, prop, strong);
      k_accept<<<div_up(L.n, B), B, 0, s>>>(L.n, prop, mate);
      count_launches(2);
    }
    uint8_t* lead = ctx.ws.get<uint8_t>(tag + ".lead", L.n);
    int32_t* lead_row = ctx.ws.get<int32_t>(tag + ".lead_row", L.n);
    k_row_lead<<<div_up(L.n, B), B, 0, s>>>(L.n, L.rp, L.cols, L.vals, active, mate, lead_row, lead);
    count_launches(1);
    int64_t* gid = ctx.ws.get<int64_t>(tag + ".gid", L.n + 1);
    exclusive_scan_u8(lead, gid, L.n, ctx.ws, s, tag + ".gs");
    const int64_t NG = read_i64(ctx, gid + L.n);
    int32_t* grp_of = ctx.ws.get<int32_t>(tag + ".grp_of", L.n);
    int32_t* gcnt = ctx.ws.get<int32_t>(tag + ".gcnt", NG);
    RUV_CUDA(cudaMemsetAsync(gcnt, 0, sizeof(int32_t) * std::max<int64_t>(NG, 1), s));
    k_group_of<<<div_up(L.n, B), B, 0, s>>>(L.n, active, lead_row, gid, grp_of, gcnt);
    count_launches(1);
    int64_t* goff = ctx.ws.get<int64_t>(tag + ".goff", NG + 1);
    exclusive_scan(gcnt, goff, NG, ctx.ws, s, tag + ".go");
    int32_t* gcur = ctx.ws.get<int32_t>(tag + ".gcur", NG);
    RUV_CUDA(cudaMemsetAsync(gcur, 0, sizeof(int32_t) * std::max<int64_t>(NG, 1), s));
    int32_t* mem = ctx.ws.get<int32_t>(tag + ".mem", L.n);
    k_group_scatter<<<div_up(L.n, B), B, 0, s>>>(L.n, active, grp_of, goff, gcur, mem);
    count_launches(1);
    int32_t* gmate = ctx.ws.get<int32_t>(tag + ".gmate", NG);
    int32_t* gprop = ctx.ws.get<int32_t>(tag + ".gprop", NG);
    int32_t* glead_of = ctx.ws.get<int32_t>(tag + ".glead_of", NG);
    uint8_t* glead = ctx.ws.get<uint8_t>(tag + ".glead", NG);
    RUV_CUDA(cudaMemsetAsync(gmate, 0xff, sizeof(int32_t) * std::max<int64_t>(NG, 1), s));
    GalWork gw;
    gw.list = ctx.ws.get<int32_t>("amg.gal_list", std::max<int64_t>(L.n, 1));
    gw.list_n = ovf + 6;
    gw.ovf = ovf;
    gw.debug = debug;
    auto mean = [](int64_t a, int64_t b) { return b > 0 ? (double)a / (double)b : 0.0; };
    if (NG > 0) {
      k_sort_members<<<div_up(NG, B), B, 0, s>>>(NG, goff, mem);
      count_launches(1);
      if (graph) {  // the group graph once, then every round and the lead pass filter it
        int32_t* gcap = ctx.ws.get<int32_t>(tag + ".gcap", NG);
        int64_t* gcap_off = ctx.ws.get<int64_t>(tag + ".gcapoff", NG + 1);
        int32_t* gn = ctx.ws.get<int32_t>(tag + ".gn", NG);
        k_group_nnz<<<div_up(NG, B), B, 0, s>>>(NG, goff, mem, L.rp, gcap);
        count_launches(1);
        exclusive_scan(gcap, gcap_off, NG, ctx.ws, s, tag + ".gcs");
        const int64_t GE = read_i64(ctx, gcap_off + NG);
        int32_t* gkey = ctx.ws.get<int32_t>("amg.gkey", std::max<int64_t>(GE, 1));
        float* gval = ctx.ws.get<float>("amg.gval", std::max<int64_t>(GE, 1));
        k_group_graph<<<div_up(NG, B), B, 0, s>>>(NG, goff, mem, L.rp, L.cols, L.vals, grp_of, gcap_off, gn, gkey, gval);
        count_launches(1);
        for (int r = 0; r < rounds; ++r) {
          k_propose2_graph<<<div_up(NG, B), B, 0, s>>>(NG, gcap_off, gn, gkey, gval, gmate, gprop, ovf, strong);
          k_accept<<<div_up(NG, B), B, 0, s>>>(NG, gprop, gmate);
          count_launches(2);
        }
        k_group_lead_graph<<<div_up(NG, B), B, 0, s>>>(NG, gcap_off, gn, gkey, gval, gmate, glead_of, glead);
        count_launches(1);
      } else {
        for (int r = 0; r < rounds; ++r) {
          k_propose2<<<div_up(NG, B), B, 0, s>>>(NG, goff, mem, L.rp, L.cols, L.vals, grp_of, gmate, gprop, ovf, strong);
          k_accept<<<div_up(NG, B), B, 0, s>>>(NG, gprop, gmate);
          count_launches(2);
        }
        k_group_lead<<<div_up(NG, B), B, 0, s>>>(NG, goff, mem, L.rp, L.cols, L.vals, grp_of, gmate, glead_of, glead);
        count_launches(1);
      }
    }
    int64_t* aid = ctx.ws.get<int64_t>(tag + ".aid", NG + 1);
    exclusive_scan_u8(glead, aid, NG, ctx.ws, s, tag + ".as");
    const int64_t NA = read_i64(ctx, aid + NG);
    int32_t* agg = ctx.ws.get<int32_t>(tag + ".agg", L.n);
    k_agg<<<div_up(L.n, B), B, 0, s>>>(L.n, active, grp_of, glead_of, aid, agg);
    L.agg = agg;
    // coarse chart offsets: aggregates are numbered in lead-row order, so chart c's
    // aggregates start at the count of aggregate-leading rows before its first row
    uint8_t* arow = ctx.ws.get<uint8_t>(tag + ".arow", L.n);
    k_agg_lead_rows<<<div_up(L.n, B), B, 0, s>>>(L.n, lead, glead, grp_of, arow);
    count_launches(2);
    int64_t* ascan = ctx.ws.get<int64_t>(tag + ".ascan", L.n + 1);
    exclusive_scan_u8(arow, ascan, L.n, ctx.ws, s, tag + ".ar");
    const std::string ntag = "amg.l" + std::to_string(lvl + 1);
    AmgLevelDev C;
    C.n = NA;
    C.chart_row = ctx.ws.get<int64_t>(ntag + ".chart_row", NC + 1);
    k_coarse_chart_rows<<<div_up(NC + 1, B), B, 0, s>>>(NC, L.chart_row, ascan, C.chart_row);
    count_launches(1);
    // ---- prolongator P (fine rows of continuing charts)
    int32_t* cnt = ctx.ws.get<int32_t>(tag + ".pcnt", L.n);
    L.poff = ctx.ws.get<int64_t>(tag + ".poff", L.n + 1);
    // one pass forms every row into a staging slot of pwid entries (a tentative row has one)
    const int pwid = sm ? pmax : 1;
    int32_t* st_pc = ctx.ws.get<int32_t>(tag + ".st_pc", L.n * pwid);
    float* st_pv = ctx.ws.get<float>(tag + ".st_pv", L.n * pwid);
    k_prolong<2><<<div_up(L.n, B), B, 0, s>>>(L.n, active, L.rp, L.cols, L.vals, L.dinv, agg, sm ? 1 : 0, pwid, cnt,
                                              nullptr, st_pc, st_pv, ovf);
    count_launches(1);
    const int64_t PN = offsets_from_counts(ctx, cnt, L.n, L.poff, tag + ".po");
    L.n_pnnz = PN;
    L.pc = ctx.ws.get<int32_t>(tag + ".pc", PN);
    L.pv = ctx.ws.get<float>(tag + ".pv", PN);
    if (L.n > 0) {
      k_prolong_copy<<<div_up(L.n, B), B, 0, s>>>(L.n, pwid, cnt, st_pc, st_pv, L.poff, L.pc, L.pv);
      count_launches(1);
    }
    // ---- R = P^T
    int32_t* rcnt = ctx.ws.get<int32_t>(tag + ".rcnt", NA);
    RUV_CUDA(cudaMemsetAsync(rcnt, 0, sizeof(int32_t) * std::max<int64_t>(NA, 1), s));
    if (PN > 0) {
      k_count_cols<<<div_up(PN, B), B, 0, s>>>(PN, L.pc, rcnt);
      count_launches(1);
    }
    L.roff = ctx.ws.get<int64_t>(tag + ".roff", NA + 1);
    exclusive_scan(rcnt, L.roff, NA, ctx.ws, s, tag + ".ro");
    int32_t* cursor = ctx.ws.get<int32_t>(tag + ".rcur", NA);
    RUV_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * std::max<int64_t>(NA, 1), s));
    L.rc = ctx.ws.get<int32_t>(tag + ".rc", PN);
    L.rv = ctx.ws.get<float>(tag + ".rv", PN);
    int32_t* rc_tmp = ctx.ws.get<int32_t>("amg.rc_tmp", PN);
    float* rv_tmp = ctx.ws.get<float>("amg.rv_tmp", PN);
    k_scatter_t<<<div_up(L.n, B), B, 0, s>>>(L.n, L.poff, L.pc, L.pv, L.roff, cursor, rc_tmp, rv_tmp);
    k_sort_rows<<<div_up(NA * 32, B), B, 0, s>>>(NA, L.roff, rc_tmp, rv_tmp, L.rc, L.rv);
    count_launches(2);
    int32_t* acnt = ctx.ws.get<int32_t>(ntag + ".acnt", NA);
    int64_t* aoff = ctx.ws.get<int64_t>(ntag + ".aoff", NA + 1);
    // the coarse operator's storage once its size is known
    auto alloc_coarse = [&](int64_t AN) {
      if (AN >= (int64_t)INT32_MAX) throw Error{RUV_ERR_BAD_INPUT, "coarse operator too large"};
      C.rp = ctx.ws.get<int32_t>(ntag + ".rp", NA + 1);
      C.cols = ctx.ws.get<int32_t>(ntag + ".cols", AN);
      C.vals = ctx.ws.get<float>(ntag + ".vals", AN);
      C.vals64 = ctx.ws.get<double>(ntag + ".vals64", AN);
      C.vals_lo = ctx.ws.get<float>(ntag + ".lo", AN);
      C.vdf = ctx.ws.get<float2>(ntag + ".vdf", AN);
      C.dinv = ctx.ws.get<float>(ntag + ".dinv", NA);
      C.nnz = AN;
    };
    auto finish_coarse = [&]() {
      if (NA > 0) {
        k_i64_i32<<<div_up(NA + 1, B), B, 0, s>>>(NA + 1, aoff, C.rp);
        if (C.nnz > 0) k_df_unpack<<<div_up(C.nnz, B), B, 0, s>>>(C.nnz, C.vdf, C.vals, C.vals_lo, C.vals64);
        count_launches(2);
      }
    };
    int64_t WN = 0;
    L.smoothed = sm;
    if (!sm) {
      // ---- tentative prolongator: A_c = R A P straight from A (keys through agg)
      const double avg = mean(PN, NA) * mean(L.nnz, L.n);
      gal_count<true>(ctx, gw, NA, avg, nullptr, L.roff, L.rc, LdOne{}, L.rp, L.cols, LdHL{L.vals, L.vals_lo},
                      KeyAgg{agg}, acnt);
      alloc_coarse(offsets_from_counts(ctx, acnt, NA, aoff, ntag + ".ao"));
      gal_fill<true>(ctx, gw, NA, L.roff, L.rc, LdOne{}, L.rp, L.cols, LdHL{L.vals, L.vals_lo}, KeyAgg{agg}, aoff,
                     C.cols, C.vdf, C.dinv);
      finish_coarse();
    } else {
      // ---- smoothed prolongator: W = A P, then A_c = R W
      int32_t* wcnt = ctx.ws.get<int32_t>(tag + ".wcnt", L.n);
      int64_t* woff = ctx.ws.get<int64_t>(tag + ".woff", L.n + 1);
      gal_count<false>(ctx, gw, L.n, mean(L.nnz, L.n) * mean(PN, L.n), active, L.rp, L.cols, LdHL{L.vals, L.vals_lo},
                       L.poff, L.pc, LdF{L.pv}, KeyId{}, wcnt);
      WN = offsets_from_counts(ctx, wcnt, L.n, woff, tag + ".wo");
      int32_t* wc = ctx.ws.get<int32_t>(tag + ".wc", WN);
      float2* wv = ctx.ws.get<float2>(tag + ".wv", WN);
      gal_fill<false>(ctx, gw, L.n, L.rp, L.cols, LdHL{L.vals, L.vals_lo}, L.poff, L.pc, LdF{L.pv}, KeyId{}, woff, wc,
                      wv, nullptr);
      gal_count<true>(ctx, gw, NA, mean(PN, NA) * mean(WN, L.n), nullptr, L.roff, L.rc, LdF{L.rv}, woff, wc, LdDF{wv},
                      KeyId{}, acnt);
      alloc_coarse(offsets_from_counts(ctx, acnt, NA, aoff, ntag + ".ao"));
      gal_fill<true>(ctx, gw, NA, L.roff, L.rc, LdF{L.rv}, woff, wc, LdDF{wv}, KeyId{}, aoff, C.cols, C.vdf, C.dinv);
      finish_coarse();
    }
    L.n_next = NA;
    if (debug) {
      int hv[8];
      RUV_CUDA(cudaMemcpyAsync(hv, ovf, sizeof(hv), cudaMemcpyDeviceToHost, s));
      RUV_CUDA(cudaStreamSynchronize(s));
      std::fprintf(stderr, "amg level %d: n=%lld nnz=%lld groups=%lld aggregates=%lld P=%lld W=%lld Ac=%lld "
                   "max keys propose2=%d P=%d W=%d Ac=%d overflow=%d\n", lvl, (long long)L.n, (long long)L.nnz,
                   (long long)NG, (long long)NA, (long long)PN, (long long)WN, (long long)C.nnz, hv[2], hv[3], hv[4], hv[5],
                   hv[0]);
      RUV_CUDA(cudaMemsetAsync(ovf + 2, 0, 4 * sizeof(int), s));
    }
    C.h_chart_row.resize(NC + 1);
    RUV_CUDA(cudaMemcpyAsync(C.h_chart_row.data(), C.chart_row, sizeof(int64_t) * (NC + 1), cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaStreamSynchronize(s));
    if (narrow) {  // 16-bit columns for the smoothers when the level allows them
      uint16_t* c16 = nullptr;
      int32_t* cbase = nullptr;
      bool rowrel = false;
      narrow_operator(ctx, NA, C.nnz, NC, C.h_chart_row, C.chart_row, C.rp, C.cols, ntag, &c16, &cbase, &rowrel);
      C.c16 = c16;
      C.cbase = cbase;
      C.rowrel = rowrel;
    }
    H->lv.push_back(C);
  }
  int h_ovf[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  RUV_CUDA(cudaMemcpyAsync(h_ovf, ovf, sizeof(h_ovf), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  if (h_ovf[0]) throw Error{RUV_ERR_INTERNAL, "AMG setup: a product row exceeded 4096 distinct columns"};
  // ---- per-level vectors, tile tables, pointer tables, dense factors
  const int NR = sys.nrhs;
  const int K = (int)H->lv.size();
  for (int k = 0; k < K; ++k) {
    AmgLevelDev& L = H->lv[k];
    const std::string tag = "amg.v" + std::to_string(k);
    const int64_t tile = level_tile_rows(k);
    for (int which = 0; which < 2; ++which) {
      std::vector<int64_t> tab, ctile(NC + 1, 0);
      std::vector<int32_t> tch;
      for (int64_t c = 0; c < NC; ++c) {
        ctile[c] = (int64_t)tch.size();
        if (which == 0 && !(H->h_final[c] > k)) continue;
        for (int64_t a0 = L.h_chart_row[c]; a0 < L.h_chart_row[c + 1]; a0 += tile) {
          tab.push_back(a0);
          tab.push_back(std::min(a0 + tile, L.h_chart_row[c + 1]));
          tch.push_back((int32_t)c);
        }
      }
      ctile[NC] = (int64_t)tch.size();
      const int64_t nt = (int64_t)tch.size();
      if (which == 0 && k < H->k_levels && nt > 0) {
        int64_t* dct = ctx.ws.get<int64_t>(tag + ".kct", NC + 1);
        RUV_CUDA(cudaMemcpyAsync(dct, ctile.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, s));
        RUV_CUDA(cudaStreamSynchronize(s));
        L.cont_chart_tile = dct;
        L.w = ctx.ws.get<float>(tag + ".kw", NR * L.n);
        L.kpart = ctx.ws.get<double>(tag + ".kpart", 2 * nt);
        L.kbeta = ctx.ws.get<float>(tag + ".kbeta", NC);
      }
      int64_t* dtab = ctx.ws.get<int64_t>(tag + (which ? ".atab" : ".ctab"), 2 * nt);
      int32_t* dch = ctx.ws.get<int32_t>(tag + (which ? ".ach" : ".cch"), nt);
      if (nt > 0) {
        RUV_CUDA(cudaMemcpyAsync(dtab, tab.data(), sizeof(int64_t) * 2 * nt, cudaMemcpyHostToDevice, s));
        RUV_CUDA(cudaMemcpyAsync(dch, tch.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice, s));
        RUV_CUDA(cudaStreamSynchronize(s));
      }
      (which ? L.all : L.cont) = LvlTiles{dtab, dch, nt};
    }
    L.b = k == 0 ? nullptr : ctx.ws.get<float>(tag + ".b", NR * L.n);
    L.x = k == 0 ? nullptr : ctx.ws.get<float>(tag + ".x", NR * L.n);
    L.y = ctx.ws.get<float>(tag + ".y", NR * L.n);
    L.t = ctx.ws.get<float>(tag + ".t", NR * L.n);
    H->total_rows += L.n;
    H->total_nnz += L.nnz;
  }
  H->final_lvl = ctx.ws.get<int32_t>("amg.final", NC);
  RUV_CUDA(cudaMemcpyAsync(H->final_lvl, H->h_final.data(), sizeof(int32_t) * NC, cudaMemcpyHostToDevice, s));
  std::vector<int64_t> foff(NC + 1, 0);
  for (int64_t c = 0; c < NC; ++c) {
    const int f = H->h_final[c];
    const int64_t m = f >= 0 ? H->lv[f].h_chart_row[c + 1] - H->lv[f].h_chart_row[c] : 0;
    foff[c + 1] = foff[c] + (m <= kDirect ? m * m : 0);
  }
  H->fac_off = ctx.ws.get<int64_t>("amg.fac_off", NC + 1);
  H->fac = ctx.ws.get<float>("amg.fac", foff[NC]);
  RUV_CUDA(cudaMemcpyAsync(H->fac_off, foff.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, s));
  std::vector<const int64_t*> cr(K);
  std::vector<const int32_t*> rps(K), cls(K);
  std::vector<const double*> vls(K);
  std::vector<const float*> dvs(K);
  for (int k = 0; k < K; ++k) {
    cr[k] = H->lv[k].chart_row;
    rps[k] = H->lv[k].rp;
    cls[k] = H->lv[k].cols;
    vls[k] = H->lv[k].vals64;
    dvs[k] = H->lv[k].dinv;
  }
  H->d_lvl_chart_row = ctx.ws.get<const int64_t*>("amg.p_cr", K);
  const int32_t** d_rp = ctx.ws.get<const int32_t*>("amg.p_rp", K);
  const int32_t** d_cols = ctx.ws.get<const int32_t*>("amg.p_cols", K);
  const double** d_vals = ctx.ws.get<const double*>("amg.p_vals", K);
  H->d_lvl_dinv = ctx.ws.get<const float*>("amg.p_dinv", K);
  RUV_CUDA(cudaMemcpyAsync(H->d_lvl_chart_row, cr.data(), sizeof(void*) * K, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_rp, rps.data(), sizeof(void*) * K, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_cols, cls.data(), sizeof(void*) * K, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_vals, vls.data(), sizeof(void*) * K, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(H->d_lvl_dinv, dvs.data(), sizeof(void*) * K, cudaMemcpyHostToDevice, s));
  int* bad = ovf + 1;
  if (NC > 0) {
    RUV_CUDA(cudaFuncSetAttribute(k_direct_factor, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFactorSmem));
    k_direct_factor<<<(unsigned)NC, kFactorThreads, kFactorSmem, s>>>(H->final_lvl, H->d_lvl_chart_row, d_rp, d_cols, d_vals, H->fac_off,
                                                 H->fac, bad);
    count_launches(1);
  }
  H->d_lvl_b = ctx.ws.get<float*>("amg.p_b", K);
  H->d_lvl_x = ctx.ws.get<float*>("amg.p_x", K);
  RUV_CUDA(cudaMemcpyAsync(h_ovf, ovf, sizeof(h_ovf), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));  // host pointer tables above go out of scope
  if (h_ovf[1]) throw Error{RUV_ERR_BREAKDOWN, "AMG setup: a coarse block is not positive definite"};
  info = "levels=" + std::to_string(K) + " rows=" + std::to_string(H->total_rows) + " nnz=" + std::to_string(H->total_nnz);
  {
    cudaEvent_t t1;
    RUV_CUDA(cudaEventCreate(&t1));
    RUV_CUDA(cudaEventRecord(t1, s));
    RUV_CUDA(cudaEventSynchronize(t1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t_setup0, t1);
    cudaEventDestroy(t1);
    if (debug) std::fprintf(stderr, "amg setup %.2f ms, %s, operator complexity %.2f\n", ms, info.c_str(),
                            sys.nnz > 0 ? (double)H->total_nnz / (double)sys.nnz : 0.0);
  }
  cudaEventDestroy(t_setup0);
  stage_setup(ctx, H.get());
  return H.release();
}

void amg_free(AmgHierarchy* H) { delete H; }

int amg_levels(const AmgHierarchy* H) { return (int)H->lv.size(); }

void amg_export_level(Ctx& ctx, const DevSystem& sys, bool smooth, int level, AmgLevelHost& out) {
  struct Free {
    void operator()(AmgHierarchy* h) const { amg_free(h); }
  };
  std::string info;
  std::unique_ptr<AmgHierarchy, Free> H(amg_setup(ctx, sys, smooth, info));
  const int K = (int)H->lv.size();
  out = AmgLevelHost();
  out.n_levels = K;
  if (level < 0 || level >= K) throw Error{RUV_ERR_BAD_INPUT, "level out of range"};
  const AmgLevelDev& L = H->lv[level];
  cudaStream_t s = ctx.stream;
  out.n = L.n;
  out.nnz = L.nnz;
  out.rp.resize(L.n + 1);
  out.cols.resize(L.nnz);
  out.vals.resize(L.nnz);
  RUV_CUDA(cudaMemcpyAsync(out.rp.data(), L.rp, sizeof(int32_t) * (L.n + 1), cudaMemcpyDeviceToHost, s));
  if (L.nnz > 0) {
    RUV_CUDA(cudaMemcpyAsync(out.cols.data(), L.cols, sizeof(int32_t) * L.nnz, cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaMemcpyAsync(out.vals.data(), L.vals64, sizeof(double) * L.nnz, cudaMemcpyDeviceToHost, s));
  }
  if (level + 1 < K && L.poff && L.agg) {
    out.smoothed = L.smoothed;
    out.n_next = H->lv[level + 1].n;
    out.pnnz = L.n_pnnz;
    out.poff.resize(L.n + 1);
    out.pc.resize(L.n_pnnz);
    out.pv.resize(L.n_pnnz);
    out.agg.resize(L.n);
    RUV_CUDA(cudaMemcpyAsync(out.poff.data(), L.poff, sizeof(int64_t) * (L.n + 1), cudaMemcpyDeviceToHost, s));
    if (L.n_pnnz > 0) {
      RUV_CUDA(cudaMemcpyAsync(out.pc.data(), L.pc, sizeof(int32_t) * L.n_pnnz, cudaMemcpyDeviceToHost, s));
      RUV_CUDA(cudaMemcpyAsync(out.pv.data(), L.pv, sizeof(float) * L.n_pnnz, cudaMemcpyDeviceToHost, s));
    }
    if (L.n > 0) RUV_CUDA(cudaMemcpyAsync(out.agg.data(), L.agg, sizeof(int32_t) * L.n, cudaMemcpyDeviceToHost, s));
  }
  RUV_CUDA(cudaStreamSynchronize(s));
}

// Bind the level-0 right-hand side / output vectors (the CG's r and z) before capture.
void amg_bind(Ctx& ctx, AmgHierarchy* H, float* r0, float* z0) {
  const int K = (int)H->lv.size();
  H->lv[0].b = r0;
  H->lv[0].x = z0;
  std::vector<float*> bs(K), xs(K);
  for (int k = 0; k < K; ++k) {
    bs[k] = H->lv[k].b;
    xs[k] = H->lv[k].x;
  }
  RUV_CUDA(cudaMemcpyAsync(H->d_lvl_b, bs.data(), sizeof(void*) * K, cudaMemcpyHostToDevice, ctx.stream));
  RUV_CUDA(cudaMemcpyAsync(H->d_lvl_x, xs.data(), sizeof(void*) * K, cudaMemcpyHostToDevice, ctx.stream));
  RUV_CUDA(cudaStreamSynchronize(ctx.stream));
}

namespace {

// Lanes per row from the operator's mean row length: one lane per row for the tentative
// prolongator (one entry per row), then enough lanes that K = 4 slots per lane cover a
// typical row in one sweep with two rows in flight (8 independent gathers per lane).
int lanes_for(double avg) { return avg <= 1.5 ? 1 : avg <= 8 ? 2 : avg <= 16 ? 4 : avg <= 32 ? 8 : 16; }

// Lanes per row of the smoothers' operator rows (A's row length): fewer lanes than the transfer
// rule, more rows per warp.  On the 4096-disk hierarchy (levels of 6.9, 15.8, 24.0 and 10.8
// entries per row) one lane per row at level 0 ran the step 1.1 ms faster than two, two lanes
// at levels 1 and 2 each 0.4 ms faster than four and eight, all together 1.6 ms (2048^2 field:
// 6.4 ms), with the same iterations.
// (RUV_AMG_SMOOTH_LANES=0: the transfer rule instead.)
int smoother_lanes(double avg) {
  const char* e = std::getenv("RUV_AMG_SMOOTH_LANES");
  if (e && e[0] == '0') return lanes_for(avg);
  return avg <= 8 ? 1 : avg <= 32 ? 2 : avg <= 64 ? 4 : avg <= 128 ? 8 : 16;
}

// Shape of the one-lane smoothers (RUV_AMG_L1SHAPE): 1 (default) = 2 rows in flight x 8
// slots, 0 = 4 x 2.  One lane sums its row in entry order whatever the shape, so both give
// the same bits; on the 4096 disks 2 x 8 ran the step 0.4 ms faster (4 x 4 was 2.5 ms slower).
int lane1_shape() {
  const char* e = std::getenv("RUV_AMG_L1SHAPE");
  return e && e[0] == '0' ? 0 : 1;
}

// Shape of the two-lane smoothers (RUV_AMG_L2SHAPE): 0 (default) = 2 rows in flight x 4 slots
// per lane, 1 = 2 x 8.  A lane sums its entries (every second one of the row) in entry order
// whatever the slot count, so both give the same bits; 2 x 8 ran the 4096-disk step 0.43 ms
// slower.
int lane2_shape() {
  const char* e = std::getenv("RUV_AMG_L2SHAPE");
  return e && e[0] == '1' ? 1 : 0;
}

#define RUV_SMOOTH_SWITCH(lpr, CALL) \
  switch (lpr) {                    \
    case 1:                         \
      if (l1s == 1) {               \
        CALL(1, 2, 8);              \
      } else {                      \
        CALL(1, 4, 2);              \
      }                             \
      break;                        \
    case 2:                         \
      if (l2s == 1) {               \
        CALL(2, 2, 8);              \
      } else {                      \
        CALL(2, 2, 4);              \
      }                             \
      break;                        \
    case 4: CALL(4, 2, 4); break;   \
    case 8: CALL(8, 2, 4); break;   \
    default: CALL(16, 1, 4); break; \
  }

// The same with a per-level override: the k-th entry of the list in `knob` (RUV_AMG_LANES for
// the smoothers, RUV_AMG_TLANES for restriction and prolongation; 0 or a missing entry: from
// the row length by `rule`; only 1, 2, 4, 8 and 16 are taken).
int lanes_at(const char* knob, int k, double avg, int (*rule)(double) = lanes_for) {
  const long long v = env_level_entry(knob, k);
  if (v == 1 || v == 2 || v == 4 || v == 8 || v == 16) return (int)v;
  return rule(avg);
}

#define RUV_LPR_SWITCH(lpr, CALL) \
  switch (lpr) {                   \
    case 1: CALL(1, 4, 2); break;  \
    case 2: CALL(2, 2, 4); break;  \
    case 4: CALL(4, 2, 4); break;  \
    case 8: CALL(8, 2, 4); break;  \
    default: CALL(16, 1, 4); break; \
  }

// The V(1,1) cycle from level k0 down: x_k0 = M^-1 b_k0 for every chart with rows at k0.
template <int NR>
int vtail(Ctx& ctx, AmgHierarchy* H, const int32_t* done, int k0) {
  cudaStream_t s = ctx.stream;
  const int l1s = lane1_shape(), l2s = lane2_shape();
  const int K = (int)H->lv.size();
  const int B = kAmgThreads;
  int launches = 0;
  for (int k = k0; k + 1 < K; ++k) {
    AmgLevelDev& L = H->lv[k];
    AmgLevelDev& C = H->lv[k + 1];
    if (L.cont.n == 0) continue;
    const int la = lanes_at("RUV_AMG_LANES", k, L.n ? (double)L.nnz / (double)L.n : 1.0, smoother_lanes);
    float* xpre = L.smoothed ? L.x : nullptr;  // the tentative cycle re-forms it on the way up
#define CALL(X, UU, KK)                                                                                                \
  if (L.stage_smem)                                                                                                    \
    k_smooth_down_st<NR, X, UU, KK, NW><<<(unsigned)L.cont.n, B, L.stage_smem, s>>>(                                   \
        L.cont, done, L.rp, L.cols, L.c16, L.cbase, L.vals, L.dinv, L.b, xpre, L.t, H->spin_limit, H->err);            \
  else                                                                                                                 \
    k_smooth_down<NR, X, UU, KK, NW><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.rp, L.cols, L.c16, L.cbase, L.vals, \
                                                                      L.dinv, L.b, xpre, L.t)
    if (L.c16 && L.rowrel) {
      constexpr int NW = 2;
      RUV_SMOOTH_SWITCH(la, CALL)
    } else if (L.c16) {
      constexpr int NW = 1;
      RUV_SMOOTH_SWITCH(la, CALL)
    } else {
      constexpr int NW = 0;
      RUV_SMOOTH_SWITCH(la, CALL)
    }
#undef CALL
    ++launches;
    if (C.all.n == 0) continue;
    const int lr = lanes_at("RUV_AMG_TLANES", k, C.n ? (double)L.n_pnnz / (double)C.n : 1.0);
#define CALL(X, UU, KK) k_restrict<NR, X, UU, KK><<<(unsigned)C.all.n, B, 0, s>>>(C.all, done, L.roff, L.rc, L.rv, L.t, C.b)
    RUV_LPR_SWITCH(lr, CALL)
#undef CALL
    ++launches;
  }
  k_direct_solve<NR><<<(unsigned)H->n_charts, kDirect, 0, s>>>(H->final_lvl, done, H->d_lvl_chart_row, H->d_lvl_b,
                                                               H->d_lvl_x, H->d_lvl_dinv, H->fac_off, H->fac, k0, kMaxLevels);
  ++launches;
  for (int k = K - 2; k >= k0; --k) {
    AmgLevelDev& L = H->lv[k];
    AmgLevelDev& C = H->lv[k + 1];
    if (L.cont.n == 0) continue;
    const int la = lanes_at("RUV_AMG_LANES", k, L.n ? (double)L.nnz / (double)L.n : 1.0, smoother_lanes);
    if (!L.smoothed) {
#define CALL(X, UU, KK)                                                                                                \
  k_smooth_up_t<NR, X, UU, KK, NW><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.rp, L.cols, L.c16, L.cbase, L.vals, \
                                                                    L.dinv, L.b, L.agg, C.x, H->alpha_c, L.x)
      if (L.c16 && L.rowrel) {
        constexpr int NW = 2;
        RUV_SMOOTH_SWITCH(la, CALL)
      } else if (L.c16) {
        constexpr int NW = 1;
        RUV_SMOOTH_SWITCH(la, CALL)
      } else {
        constexpr int NW = 0;
        RUV_SMOOTH_SWITCH(la, CALL)
      }
#undef CALL
      ++launches;
      continue;
    }
    const int lp = lanes_at("RUV_AMG_TLANES", k, L.n ? (double)L.n_pnnz / (double)L.n : 1.0);
#define CALL(X, UU, KK)                                                                                                  \
  k_prolong_add<NR, X, UU, KK><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.poff, L.pc, L.pv, C.x, L.x, L.y, 1.0f)
    RUV_LPR_SWITCH(lp, CALL)
#undef CALL
#define CALL(X, UU, KK)                                                                                              \
  if (L.stage_smem)                                                                                                  \
    k_smooth_up_st<NR, X, UU, KK, NW><<<(unsigned)L.cont.n, B, L.stage_smem, s>>>(                                   \
        L.cont, done, L.rp, L.cols, L.c16, L.cbase, L.vals, L.dinv, L.b, L.y, L.x, H->spin_limit, H->err);           \
  else                                                                                                               \
    k_smooth_up<NR, X, UU, KK, NW><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.rp, L.cols, L.c16, L.cbase, L.vals, \
                                                                    L.dinv, L.b, L.y, L.x)
    if (L.c16 && L.rowrel) {
      constexpr int NW = 2;
      RUV_SMOOTH_SWITCH(la, CALL)
    } else if (L.c16) {
      constexpr int NW = 1;
      RUV_SMOOTH_SWITCH(la, CALL)
    } else {
      constexpr int NW = 0;
      RUV_SMOOTH_SWITCH(la, CALL)
    }
#undef CALL
    launches += 2;
  }
  return launches;
}

template <int NR>
int cycle(Ctx& ctx, AmgHierarchy* H, const int32_t* done, int k);

// Level k in the K-form (gpu/src/amg.rs:468-639), for the charts that continue below it:
// pre-smoothing from zero (x = w D^-1 b, t = b - A x), then two coarse corrections
// y = P (cycle of level k + 1 on R t), each scaled by its CG steplength
// beta = (y.t) / (y.A y) per chart (x += beta y; the first also t -= beta A y), no
// post-smoothing.  Charts whose last level is k get their direct solve.
template <int NR>
int kform(Ctx& ctx, AmgHierarchy* H, const int32_t* done, int k) {
  cudaStream_t s = ctx.stream;
  const int B = kAmgThreads;
  AmgLevelDev& L = H->lv[k];
  AmgLevelDev& C = H->lv[k + 1];
  int launches = 0;
  const int l1s = lane1_shape(), l2s = lane2_shape();
  const int la = lanes_at("RUV_AMG_LANES", k, L.n ? (double)L.nnz / (double)L.n : 1.0, smoother_lanes);
#define CALL(X, UU, KK)                                                                                                \
  k_smooth_down<NR, X, UU, KK, NW><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.rp, L.cols, L.c16, L.cbase, L.vals, \
                                                                    L.dinv, L.b, L.x, L.t)
  if (L.c16 && L.rowrel) {
    constexpr int NW = 2;
    RUV_SMOOTH_SWITCH(la, CALL)
  } else if (L.c16) {
    constexpr int NW = 1;
    RUV_SMOOTH_SWITCH(la, CALL)
  } else {
    constexpr int NW = 0;
    RUV_SMOOTH_SWITCH(la, CALL)
  }
#undef CALL
  ++launches;
  const int lr = lanes_for(C.n ? (double)L.n_pnnz / (double)C.n : 1.0);
  const int lp = lanes_for(L.n ? (double)L.n_pnnz / (double)L.n : 1.0);
  for (int step = 0; step < 2; ++step) {
#define CALL(X, UU, KK) k_restrict<NR, X, UU, KK><<<(unsigned)C.all.n, B, 0, s>>>(C.all, done, L.roff, L.rc, L.rv, L.t, C.b)
    RUV_LPR_SWITCH(lr, CALL)
#undef CALL
    ++launches;
    launches += cycle<NR>(ctx, H, done, k + 1);
#define CALL(X, UU, KK)                                                                                                  \
  k_prolong_add<NR, X, UU, KK><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.poff, L.pc, L.pv, C.x, nullptr, L.y, 1.0f)
    RUV_LPR_SWITCH(lp, CALL)
#undef CALL
#define CALL(X, UU, KK)                                                                                           \
  k_kspmv<NR, X, UU, KK, NW><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.rp, L.cols, L.c16, L.cbase, L.vals, L.y, \
                                                              L.t, L.w, L.kpart)
    if (L.c16 && L.rowrel) {
      constexpr int NW = 2;
      RUV_SMOOTH_SWITCH(la, CALL)
    } else if (L.c16) {
      constexpr int NW = 1;
      RUV_SMOOTH_SWITCH(la, CALL)
    } else {
      constexpr int NW = 0;
      RUV_SMOOTH_SWITCH(la, CALL)
    }
#undef CALL
    k_kbeta<<<(unsigned)H->n_charts, 128, 0, s>>>(done, L.cont_chart_tile, L.kpart, L.kbeta);
    k_kupdate<NR><<<(unsigned)L.cont.n, B, 0, s>>>(L.cont, done, L.kbeta, L.y, L.w, L.x, step == 0 ? L.t : nullptr);
    launches += 4;
  }
  k_direct_solve<NR><<<(unsigned)H->n_charts, kDirect, 0, s>>>(H->final_lvl, done, H->d_lvl_chart_row, H->d_lvl_b,
                                                               H->d_lvl_x, H->d_lvl_dinv, H->fac_off, H->fac, k, k);
  return launches + 1;
}

template <int NR>
int cycle(Ctx& ctx, AmgHierarchy* H, const int32_t* done, int k) {
  const int K = (int)H->lv.size();
  if (k < H->k_levels && k + 1 < K && H->lv[k].cont.n > 0 && H->lv[k].kbeta) return kform<NR>(ctx, H, done, k);
  return vtail<NR>(ctx, H, done, k);
}

}  // namespace

// One cycle (V(1,1), or the K-form on the top RUV_AMG_KCYCLE levels): z0 = M^-1 r0 for every
// chart not marked done (launches only; capturable).
int amg_apply(Ctx& ctx, AmgHierarchy* H, const int32_t* done) {
  return H->nrhs == 2 ? cycle<2>(ctx, H, done, 0) : cycle<1>(ctx, H, done, 0);
}

namespace {
// The V-cycle runs in FP32 under either CG loop; it varies slightly between applications
// (FP32 rounding, the coarse over-correction), so the CG uses the flexible beta.
class AmgPrecond final : public SepPrecond {
 public:
  AmgPrecond(Ctx& ctx, const DevSystem& sys, bool smooth) {
    std::string info;
    H_ = amg_setup(ctx, sys, smooth, info);
  }
  ~AmgPrecond() override { amg_free(H_); }
  bool native_fp64() const override { return false; }
  bool flexible() const override { return true; }
  void bind(Ctx& ctx, void* r, void* z, bool) override { amg_bind(ctx, H_, static_cast<float*>(r), static_cast<float*>(z)); }
  int apply(Ctx& ctx, const int32_t* done) override { return amg_apply(ctx, H_, done); }
  const int* error_flag() const override { return H_->err; }

 private:
  AmgHierarchy* H_ = nullptr;
};
}  // namespace

std::unique_ptr<SepPrecond> make_amg(Ctx& ctx, const DevSystem& sys, bool smooth) {
  return std::unique_ptr<SepPrecond>(new AmgPrecond(ctx, sys, smooth));
}

}  // namespace ruv
