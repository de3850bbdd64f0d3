// rd_pair.cuh -- the pair-sum engine shared by the force, field and
// Metropolis-Hastings kernels.
//
// A pair sum (particles or surface points i against the particles j of the
// same diode) is cut into work items: an i-tile of RD_ITILE consecutive i
// times a j-chunk of consecutive particles.  A plan (one entry per diode,
// built on the device from the particle counts) says how many tiles and
// chunks each diode has; persistent CTAs walk the item index space
// (round-robin, or drawing items from a counter: queue_first / queue_next)
// and decode
// (diode, tile, chunk) by binary search.  When a tile
// has more than one chunk, each chunk stores its partial sums in scratch and
// the last chunk to finish (an atomic ticket, no waiting) adds the partials
// in chunk order, so results do not depend on scheduling.
#pragma once
#include <mutex>
#include <unordered_map>
#include "rd_device.cuh"

// Persistent grid size: a positive request wins; otherwise every SM gets as
// many CTAs as can be resident at once (occupancy API), cached per kernel.
template <class F>
inline int rd_grid(F kernel, int block, int requested) {
  if (requested > 0) return requested;
  static std::mutex mu;
  static std::unordered_map<const void*, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find((const void*)kernel);
  if (it != cache.end()) return it->second;
  int dev = 0, sms = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0) != cudaSuccess || per < 1)
    per = 1;
  const int g = sms * per;
  cache[(const void*)kernel] = g;
  return g;
}

struct PlanEntry {
  int item_off;   // first item of this diode
  int tiles;      // i-tiles
  int nch;        // j-chunks per tile
  int clen;       // j-chunk length (multiple of RD_TILE)
  int n_i;        // number of i (particles or points)
  int n_j;        // number of j particles
  int pad0;       // MH plans: first global chain index of the diode
  int tsize;      // i-tile width (RD_ITILE for pair sums, 1024 for compaction)
};

struct PlanHeader {
  int total_items;
  int n_diodes;    // entries in the plan
  int pad[2];
};

struct ItemRef {
  int d;        // plan entry (== diode slot)
  int tile, chunk, nch;
  int i0, j0, j1;
  int base;     // item index of chunk 0 of this tile (partial / ticket slot)
};

__device__ __forceinline__ ItemRef decode_item(const PlanEntry* plan, int nd, int g) {
  int lo = 0, hi = nd - 1;
  while (lo < hi) {   // last entry with item_off <= g
    int mid = (lo + hi + 1) >> 1;
    if (plan[mid].item_off <= g) lo = mid; else hi = mid - 1;
  }
  const PlanEntry& e = plan[lo];
  ItemRef r;
  r.d = lo;
  int local = g - e.item_off;
  r.tile = local / e.nch;
  r.chunk = local - r.tile * e.nch;
  r.nch = e.nch;
  r.i0 = r.tile * e.tsize;
  r.j0 = r.chunk * e.clen;
  r.j1 = min(r.j0 + e.clen, e.n_j);
  r.base = e.item_off + r.tile * e.nch;
  return r;
}

// Stores this CTA's partials, then returns true in the CTA that completed
// the tile (all chunks stored).  ncomp doubles per i, layout
// partial[(item * ncomp + c) * RD_ITILE + tid].
__device__ __forceinline__ bool tile_ticket(int* tickets, const ItemRef& it) {
  __shared__ int s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    int prev = atomicAdd(&tickets[it.base], 1);
    s_last = (prev == it.nch - 1);
    if (s_last) tickets[it.base] = 0;   // reset for the next launch
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0;
}

// Dynamic item scheduling over the item range [lo, hi) of a launch.  The
// P = min(grid, hi - lo) first blocks take items lo..lo+P-1 (the others exit
// at once); after that a block draws its next item from a counter
// (lo + P + q[0]++) instead of walking a fixed stride, so blocks that drew
// cheap items (small diodes) take more and the launch ends with the work, not
// with the unluckiest block.  The last of the P blocks to leave (q[1]) resets
// both counters for the next launch on the stream; its fence orders each
// block's last draw before its leave.  No block waits on another; results do
// not depend on the order (partials are added in chunk order by tile_ticket).
__device__ __forceinline__ int queue_first(int lo, int hi) {
  return lo + (int)blockIdx.x < hi ? lo + (int)blockIdx.x : hi;
}

__device__ __forceinline__ int queue_next(int* q, int* s_slot, int lo, int hi) {
  const int P = min((int)gridDim.x, hi - lo);
  __syncthreads();
  if (threadIdx.x == 0) *s_slot = lo + P + atomicAdd(&q[0], 1);
  __syncthreads();
  return *s_slot;
}

__device__ __forceinline__ void queue_leave(int* q, int lo, int hi) {
  const int P = min((int)gridDim.x, hi - lo);
  if ((int)blockIdx.x >= P) return;   // took no item
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&q[1], 1) == P - 1) {
      q[0] = 0;
      q[1] = 0;
      __threadfence();
    }
  }
}

// Item range of one part of a plan: part 0 is the whole plan; parts
// 1..nparts cut it at the diode boundaries nearest to k/nparts of the items,
// so that nparts launches on as many streams (each with its own item
// counters) share the GPU and fill the SMs that the others' last items leave
// idle.  Every diode's items stay in one part; all parts compute the same cuts.
__device__ __forceinline__ int part_cut(const PlanEntry* plan, int nd, int total, int k, int nparts) {
  if (k <= 0) return 0;
  if (k >= nparts) return total;
  const int target = (int)(((long long)total * k) / nparts);
  int a = 0, b = nd - 1;   // last entry with item_off <= target
  while (a < b) {
    const int mid = (a + b + 1) >> 1;
    if (plan[mid].item_off <= target) a = mid; else b = mid - 1;
  }
  const int below = min(plan[a].item_off, total);
  const int above = a + 1 < nd ? min(plan[a + 1].item_off, total) : total;
  return (target - below <= above - target) ? below : above;
}

__device__ __forceinline__ void part_range(const PlanEntry* plan, int nd, int total, int part, int nparts,
                                           int* lo, int* hi) {
  if (part == 0 || nd == 0) { *lo = 0; *hi = part == 0 ? total : 0; return; }
  *lo = part_cut(plan, nd, total, part - 1, nparts);
  *hi = part_cut(plan, nd, total, part, nparts);
}

// Points of a field evaluation: per-diode lists at [off[d], off[d] + n_d).
struct PointSet {   // per-diode point lists at [pt_off_d, pt_off_d + n_d)
  const double *x, *y, *z;
  double *fx, *fy, *fz;
  const int* off;   // per diode slot
};
