// Track ordering for the navigation step: a key per track (logical volume of the current
// state in the high bits, Morton code of the position cell in the low bits) and a stable
// LSD radix sort of (key, track index) pairs with 8-bit digits. The step kernels then walk
// tracks in key order, so a warp's 32 lanes share the mother shape, the BVH and mostly the
// BVH path. The sort only permutes work: every track's result is computed exactly as in
// the unsorted launch and written at the track's own index. Digits are 9 bits wide (512
// buckets), so the 26-bit keys of the tuned detector sort (7 Morton bits per axis beside the
// logical volume) take three passes instead of four.
#include "launch.h"

namespace vg {
namespace {

constexpr int kSortBlock = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile  = kSortBlock * kSortItems;
constexpr int kSortWarps = kSortBlock / 32;
constexpr int kDigitBits = 9;
constexpr int kRadix     = 1 << kDigitBits; // buckets per pass: two per thread of a block
static_assert(kRadix == 2 * kSortBlock, "each thread scans two digits");

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

__device__ __forceinline__ uint32_t spread3(uint32_t v) // 10 bits -> every third bit
{
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__device__ __forceinline__ uint32_t cell(double c, float lo, float scale, uint32_t maxc)
{
  const float f = ((float)c - lo) * scale;
  if (!(f > 0.f)) return 0u; // also NaN
  return f >= (float)maxc ? maxc : (uint32_t)f;
}

__global__ void __launch_bounds__(256) k_sort_keys(const DevGeom g, const SortKeyParams p, const double *__restrict__ x,
                                                   const double *__restrict__ y, const double *__restrict__ z,
                                                   const NavState *__restrict__ in, const uint32_t *__restrict__ list,
                                                   size_t begin, size_t end, uint32_t *__restrict__ keys,
                                                   const unsigned int *__restrict__ n_dev)
{
  if (n_dev && begin + *n_dev < end) end = begin + *n_dev;
  const uint32_t maxc = (1u << p.cell_bits) - 1u;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t j = begin + (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < end; j += stride) {
    const size_t i     = list ? (size_t)__ldg(list + j) : j;
    const uint32_t nav = in[i].navInd;
    uint32_t key       = 0xffffffffu; // outside the world or not a table node: last
    if (nav != 0u && nav + 2u < g.nav_words) {
      const uint32_t pv = __ldg(&g.nav[nav + 1]);
      if (pv < (uint32_t)g.n_pv) {
        const uint32_t lv = (uint32_t)__ldg(&g.pv_lv[pv]);
        const uint32_t m  = spread3(cell(__ldg(x + i), p.lo[0], p.scale[0], maxc)) |
                           (spread3(cell(__ldg(y + i), p.lo[1], p.scale[1], maxc)) << 1) |
                           (spread3(cell(__ldg(z + i), p.lo[2], p.scale[2], maxc)) << 2);
        key = (lv << (3 * p.cell_bits)) | m;
      }
    }
    keys[j] = key;
  }
}

// Per-tile digit counts, digit-major: hist[d * ntiles + tile].
__global__ void __launch_bounds__(kSortBlock) k_radix_hist(const uint32_t *__restrict__ keys, size_t n, int shift,
                                                           uint32_t *__restrict__ hist, unsigned ntiles,
                                                           const unsigned int *__restrict__ n_dev)
{
  if (n_dev && *n_dev < n) n = *n_dev;
  __shared__ uint32_t h[kRadix];
  for (int k = threadIdx.x; k < kRadix; k += kSortBlock) h[k] = 0u;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i    = base + (size_t)r * kSortBlock + threadIdx.x;
    const uint32_t d  = i < n ? (__ldg(keys + i) >> shift) & (kRadix - 1u) : (uint32_t)kRadix;
    const uint32_t pm = __match_any_sync(0xffffffffu, d);
    if (d < (uint32_t)kRadix && (pm & ((1u << (threadIdx.x & 31)) - 1u)) == 0u) atomicAdd(&h[d], (uint32_t)__popc(pm));
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kRadix; k += kSortBlock) hist[(size_t)k * ntiles + blockIdx.x] = h[k];
}

// Exclusive block-wide scan of one value per thread (blockDim.x a multiple of 32, <= 1024);
// returns the exclusive prefix and leaves the block total in *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *wsum, uint32_t *total)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const uint32_t x = lane < nw ? wsum[lane] : 0u;
    uint32_t ix      = x;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, ix, o);
      if (lane >= o) ix += t;
    }
    if (lane < nw) wsum[lane] = ix - x;
    if (lane == 31) wsum[32] = ix;
  }
  __syncthreads();
  const uint32_t r = wsum[w] + incl - v;
  *total           = wsum[32];
  __syncthreads();
  return r;
}

// Row d of the digit-major counts: exclusive scan over the tiles in place (one block per
// digit); the row total goes to totals[d].
__global__ void __launch_bounds__(1024) k_scan_rows(uint32_t *__restrict__ hist, unsigned ntiles,
                                                    uint32_t *__restrict__ totals)
{
  __shared__ uint32_t wsum[33];
  uint32_t *row = hist + (size_t)blockIdx.x * ntiles;
  uint32_t carry = 0u;
  for (unsigned c = 0; c < ntiles; c += blockDim.x) {
    const unsigned i = c + threadIdx.x;
    const uint32_t v = i < ntiles ? row[i] : 0u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(v, wsum, &tot);
    if (i < ntiles) row[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

// Stable scatter of one digit. Tile positions are (warp, round, lane) in that order, so
// ranks follow the input order within a tile; tiles are ordered by the scanned counts.
__global__ void __launch_bounds__(kSortBlock) k_radix_scatter(const uint32_t *__restrict__ kin,
                                                              const uint32_t *__restrict__ vin,
                                                              uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                              size_t n, int shift, const uint32_t *__restrict__ hist,
                                                              const uint32_t *__restrict__ totals, unsigned ntiles,
                                                              const uint32_t *__restrict__ list,
                                                              const unsigned int *__restrict__ n_dev)
{
  if (n_dev && *n_dev < n) n = *n_dev;
  __shared__ uint32_t cnt[kSortWarps][kRadix];
  __shared__ uint32_t wsum[33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < kSortWarps * kRadix; k += kSortBlock) (&cnt[0][0])[k] = 0u;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kSortTile + (size_t)w * (32 * kSortItems);
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i  = base + (size_t)r * 32 + lane;
    const bool ok   = i < n;
    key[r]          = ok ? __ldg(kin + i) : 0u;
    val[r]          = ok ? (vin ? __ldg(vin + i) : (list ? __ldg(list + i) : (uint32_t)i)) : 0u;
    const uint32_t d  = ok ? (key[r] >> shift) & (kRadix - 1u) : (uint32_t)kRadix;
    const uint32_t pm = __match_any_sync(0xffffffffu, d);
    const uint32_t before = ok ? cnt[w][d] : 0u;
    __syncwarp();
    if (ok && (pm & lt) == 0u) cnt[w][d] = before + (uint32_t)__popc(pm);
    __syncwarp();
    rank[r] = before + (uint32_t)__popc(pm & lt);
  }
  __syncthreads();
  {
    // digits 2t and 2t + 1: their start = the totals of all lower digits + this row's
    // count in the tiles before this one, then each warp's share in warp order
    const uint32_t d0 = 2u * threadIdx.x, d1 = d0 + 1u;
    const uint32_t t0 = __ldg(totals + d0), t1 = __ldg(totals + d1);
    uint32_t tot;
    const uint32_t below = block_exclusive_scan(t0 + t1, wsum, &tot);
    uint32_t run0        = below + __ldg(hist + (size_t)d0 * ntiles + blockIdx.x);
    uint32_t run1        = below + t0 + __ldg(hist + (size_t)d1 * ntiles + blockIdx.x);
    for (int ww = 0; ww < kSortWarps; ++ww) {
      const uint32_t c0 = cnt[ww][d0], c1 = cnt[ww][d1];
      cnt[ww][d0]       = run0;
      cnt[ww][d1]       = run1;
      run0 += c0;
      run1 += c1;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i = base + (size_t)r * 32 + lane;
    if (i < n) {
      const uint32_t pos = cnt[w][(key[r] >> shift) & (kRadix - 1u)] + rank[r];
      kout[pos]          = key[r];
      vout[pos]          = val[r];
    }
  }
}

inline unsigned grid_for(size_t n, int block)
{
  size_t blocks       = (n + block - 1) / block;
  const size_t maxgrd = 152 * 16;
  if (blocks > maxgrd) blocks = maxgrd;
  return (unsigned)(blocks ? blocks : 1);
}

} // namespace

size_t nav_sort_workspace_bytes(size_t n)
{
  const size_t ntiles = (n + kSortTile - 1) / kSortTile;
  return 4 * align256(n * sizeof(uint32_t)) + align256(kRadix * ntiles * sizeof(uint32_t)) + kRadix * sizeof(uint32_t);
}

const uint32_t *nav_sort_keys_of(const uint32_t *order, const void *ws, size_t n)
{
  // buffers: k0, k1, v0, v1 (each align256(4n)); values in v0 pair with keys in k1
  const unsigned char *w = static_cast<const unsigned char *>(ws);
  const size_t a         = align256(n * sizeof(uint32_t));
  return reinterpret_cast<const uint32_t *>(order == reinterpret_cast<const uint32_t *>(w + 2 * a) ? w + a : w);
}

int sort_key_bits(const SortKeyParams &p) { return p.lv_bits + 3 * p.cell_bits; }

cudaError_t launch_nav_sort_keys(const DevGeom &g, const SortKeyParams &p, const double *x, const double *y,
                                 const double *z, const NavState *in, size_t begin, size_t end, void *ws,
                                 cudaStream_t s)
{
  if (end <= begin) return cudaSuccess;
  k_sort_keys<<<grid_for(end - begin, 256), 256, 0, s>>>(g, p, x, y, z, in, nullptr, begin, end,
                                                        static_cast<uint32_t *>(ws), nullptr);
  return cudaGetLastError();
}

cudaError_t launch_nav_sort(const DevGeom &g, const SortKeyParams &p, const double *x, const double *y,
                            const double *z, const NavState *in, size_t n, void *ws, const uint32_t **order,
                            cudaStream_t s, const uint32_t *list, bool keys_done, const unsigned int *n_dev)
{
  *order = nullptr;
  if (n == 0) return cudaSuccess;
  const unsigned ntiles = (unsigned)((n + kSortTile - 1) / kSortTile);
  unsigned char *w      = static_cast<unsigned char *>(ws);
  const size_t a        = align256(n * sizeof(uint32_t));
  uint32_t *k0 = reinterpret_cast<uint32_t *>(w), *k1 = reinterpret_cast<uint32_t *>(w + a);
  uint32_t *v0 = reinterpret_cast<uint32_t *>(w + 2 * a), *v1 = reinterpret_cast<uint32_t *>(w + 3 * a);
  uint32_t *hist   = reinterpret_cast<uint32_t *>(w + 4 * a);
  uint32_t *totals = reinterpret_cast<uint32_t *>(w + 4 * a + align256(kRadix * (size_t)ntiles * sizeof(uint32_t)));
  if (!keys_done) k_sort_keys<<<grid_for(n, 256), 256, 0, s>>>(g, p, x, y, z, in, list, 0, n, k0, n_dev);
  // Digits above the key's width are all zero (invalid states carry all-ones keys, which
  // sort last within every pass), so only the passes that cover the key bits are run.
  const int bits   = sort_key_bits(p);
  const int passes = (bits + kDigitBits - 1) / kDigitBits;
  uint32_t *kin = k0, *kout = k1, *vin = nullptr, *vout = v0;
  for (int ps = 0; ps < passes; ++ps) {
    k_radix_hist<<<ntiles, kSortBlock, 0, s>>>(kin, n, kDigitBits * ps, hist, ntiles, n_dev);
    k_scan_rows<<<kRadix, 1024, 0, s>>>(hist, ntiles, totals);
    k_radix_scatter<<<ntiles, kSortBlock, 0, s>>>(kin, vin, kout, vout, n, kDigitBits * ps, hist, totals, ntiles,
                                                  list, n_dev);
    uint32_t *tk = kin;
    kin          = kout;
    kout         = tk;
    vin          = vout;
    vout         = (vout == v0) ? v1 : v0;
  }
  *order = passes > 0 ? vin : nullptr;
  return cudaGetLastError();
}

} // namespace vg
