// Device RAS set-up of one level (domain division, coarse points) as segmented sorts.
//
// Every domain of a division generation, and every cluster of a coarse-point generation, is a
// segment of one element array (an element is a position k in the level's point list). A
// generation sorts all its segments at once by (segment, rank on the segment's widest axis,
// rank on the second, rank on the third): two stable radix sorts over dense per-axis ranks of
// the level's coordinates, whose lexicographic order is that of the coordinates (the reference
// orders the axes by decreasing bbox width and compares lexicographically,
// domain_divider.hpp:192-196). A segment's children are then slices of its sorted order. The
// split positions depend only on a segment's size, so the host plans a whole division from
// the sizes and launches it without round trips; the coarse-point selection reads back the
// cluster order only in its last generation, which accepts part of the splits.
#include "ras_divide.hpp"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>
#include <bit>
#include <utility>

#include "ras_host.hpp"

namespace pgpu {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// Order-preserving unsigned image of a double; -0 and +0 map to the same key.
__device__ __forceinline__ uint64_t ordered_key(double x) {
  if (x == 0.0) x = 0.0;
  const uint64_t u = static_cast<uint64_t>(__double_as_longlong(x));
  return (u >> 63) ? ~u : (u | (uint64_t{1} << 63));
}

__device__ __forceinline__ Index thread_index() {
  return static_cast<Index>(blockIdx.x) * blockDim.x + threadIdx.x;
}

// x[a n + k] = coordinate a of the level's k-th point.
__global__ void gather_coords_kernel(const double* __restrict__ pts, const Index* __restrict__ idx,
                                     Index n, double* __restrict__ x) {
  const Index k = thread_index();
  if (k >= n) return;
  const Index i = idx[k];
  for (int a = 0; a < 3; ++a) x[a * n + k] = pts[3 * i + a];
}

__global__ void axis_keys_kernel(const double* __restrict__ x, Index n, uint64_t* __restrict__ key,
                                 int* __restrict__ val) {
  const Index k = thread_index();
  if (k >= n) return;
  key[k] = ordered_key(x[k]);
  val[k] = static_cast<int>(k);
}

__global__ void new_value_flags_kernel(const uint64_t* __restrict__ skey, Index n,
                                       unsigned* __restrict__ f) {
  const Index t = thread_index();
  if (t >= n) return;
  f[t] = (t > 0 && skey[t] != skey[t - 1]) ? 1u : 0u;
}

// rank[k] = dense rank of x[k] on its axis; uq[r] = the coordinate of rank r (zeros positive).
__global__ void rank_scatter_kernel(const unsigned* __restrict__ r, const int* __restrict__ sval,
                                    const double* __restrict__ x, Index n, unsigned* __restrict__ rank,
                                    double* __restrict__ uq) {
  const Index t = thread_index();
  if (t >= n) return;
  const int k = sval[t];
  const unsigned rk = r[t];
  rank[k] = rk;
  const double v = x[k];
  uq[rk] = v == 0.0 ? 0.0 : v;
}

// Per-segment bbox in rank space: mn/mx[a S + s]. A warp whose elements share one segment
// reduces first and issues one atomic per axis.
__global__ void seg_bbox_kernel(const int* __restrict__ el_k, const int* __restrict__ el_seg,
                                Index m, const unsigned* __restrict__ rank, Index n, int S,
                                unsigned* __restrict__ mn, unsigned* __restrict__ mx) {
  const Index i = thread_index();
  if (i - static_cast<Index>(threadIdx.x & 31) >= m) return;  // the whole warp is past the end
  const bool valid = i < m;
  const int s = valid ? el_seg[i] : -1;
  const int s0 = __shfl_sync(kFull, s, 0);
  const bool uniform = __all_sync(kFull, !valid || s == s0);
  const int k = valid ? el_k[i] : 0;
  for (int a = 0; a < 3; ++a) {
    const unsigned r = valid ? rank[a * n + k] : 0u;
    if (uniform) {
      const unsigned lo = __reduce_min_sync(kFull, valid ? r : 0xffffffffu);
      const unsigned hi = __reduce_max_sync(kFull, valid ? r : 0u);
      if ((threadIdx.x & 31) == 0) {
        atomicMin(mn + static_cast<Index>(a) * S + s0, lo);
        atomicMax(mx + static_cast<Index>(a) * S + s0, hi);
      }
    } else if (valid) {
      atomicMin(mn + static_cast<Index>(a) * S + s, r);
      atomicMax(mx + static_cast<Index>(a) * S + s, r);
    }
  }
}

// Axes by decreasing bbox width, equal widths in axis order (the stable order std::sort gives
// three elements); packed a0 | a1 << 2 | a2 << 4. Optionally the bbox volume and centre, with
// the host's roundings: (w0 w1) w2 and min + w / 2.
__global__ void seg_shape_kernel(int S, const unsigned* __restrict__ mn,
                                 const unsigned* __restrict__ mx, const double* __restrict__ uq,
                                 Index n, unsigned char* __restrict__ axes,
                                 double* __restrict__ volume, double* __restrict__ ctr) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  double lo[3], w[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = uq[a * n + mn[static_cast<Index>(a) * S + s]];
    w[a] = __dsub_rn(uq[a * n + mx[static_cast<Index>(a) * S + s]], lo[a]);
  }
  int ax[3] = {0, 1, 2};
  for (int i = 1; i < 3; ++i)
    for (int j = i; j > 0 && w[ax[j - 1]] < w[ax[j]]; --j) {
      const int t = ax[j];
      ax[j] = ax[j - 1];
      ax[j - 1] = t;
    }
  axes[s] = static_cast<unsigned char>(ax[0] | (ax[1] << 2) | (ax[2] << 4));
  if (volume) volume[s] = __dmul_rn(__dmul_rn(w[0], w[1]), w[2]);
  if (ctr)
    for (int a = 0; a < 3; ++a) ctr[static_cast<Index>(a) * S + s] = __dadd_rn(lo[a], __dmul_rn(w[a], 0.5));
}

// Pass 1 keys: (rank on the second axis, rank on the third) of each element's segment.
__global__ void minor_keys_kernel(const int* __restrict__ el_k, const int* __restrict__ el_seg,
                                  Index m, const unsigned* __restrict__ rank, Index n,
                                  const unsigned char* __restrict__ axes, int b,
                                  uint64_t* __restrict__ key, int* __restrict__ val) {
  const Index i = thread_index();
  if (i >= m) return;
  const unsigned ax = axes[el_seg[i]];
  const int k = el_k[i];
  key[i] = (static_cast<uint64_t>(rank[((ax >> 2) & 3) * n + k]) << b) | rank[((ax >> 4) & 3) * n + k];
  val[i] = static_cast<int>(i);
}

// Pass 2 keys, in pass 1 order: (segment, rank on the first axis).
__global__ void major_keys_kernel(const int* __restrict__ order, const int* __restrict__ el_k,
                                  const int* __restrict__ el_seg, Index m,
                                  const unsigned* __restrict__ rank, Index n,
                                  const unsigned char* __restrict__ axes, int b,
                                  uint64_t* __restrict__ key, int* __restrict__ val) {
  const Index t = thread_index();
  if (t >= m) return;
  const int i = order[t];
  const int s = el_seg[i];
  key[t] = (static_cast<uint64_t>(s) << b) | rank[(axes[s] & 3) * n + el_k[i]];
  val[t] = i;
}

// A splitting domain of one division generation.
struct DivSeg {
  Index begin, n, left_part, mid, right_part;
  Index dst[2];  // first element of each child in its destination array
  int id[2];     // the child's segment in the next generation, or its domain (leaf)
  int leaf[2];   // 1: the child is a leaf
};

__global__ void init_elements_kernel(Index m, int* __restrict__ k, unsigned char* __restrict__ in,
                                     int* __restrict__ seg) {
  const Index t = thread_index();
  if (t >= m) return;
  k[t] = static_cast<int>(t);
  in[t] = 1;
  seg[t] = 0;
}

// Writes both overlapping halves of every sorted domain (domain_divider.hpp:214-248).
__global__ void div_scatter_kernel(const int* __restrict__ perm, Index m, const int* __restrict__ el_k,
                                   const unsigned char* __restrict__ el_in,
                                   const int* __restrict__ el_seg, const DivSeg* __restrict__ segs,
                                   int* __restrict__ nk, unsigned char* __restrict__ nin,
                                   int* __restrict__ nseg, int* __restrict__ lk,
                                   unsigned char* __restrict__ lin, int* __restrict__ ldom) {
  const Index t = thread_index();
  if (t >= m) return;
  const int i = perm[t];
  const DivSeg& g = segs[el_seg[i]];
  const Index r = t - g.begin;
  const int k = el_k[i];
  const bool in = el_in[i] != 0;
  for (int c = 0; c < 2; ++c) {
    if (c == 0 ? r >= g.right_part : r < g.left_part) continue;
    const Index pos = g.dst[c] + (c == 0 ? r : r - g.left_part);
    const unsigned char inner = (in && (c == 0 ? r < g.mid : r >= g.mid)) ? 1 : 0;
    if (g.leaf[c]) {
      lk[pos] = k;
      lin[pos] = inner;
      ldom[pos] = g.id[c];
    } else {
      nk[pos] = k;
      nin[pos] = inner;
      nseg[pos] = g.id[c];
    }
  }
}

// Domain::merge_poly_points (domain.hpp:27-49) keys: (domain, polynomial slot) for the
// polynomial points (positions k < np of the level), (domain, 1, global index) for the rest.
__global__ void merge_keys_kernel(const int* __restrict__ lk, const int* __restrict__ ldom, Index m,
                                  int np, const Index* __restrict__ gidx, int bits,
                                  uint64_t* __restrict__ key, int* __restrict__ val,
                                  int* __restrict__ present) {
  const Index e = thread_index();
  if (e >= m) return;
  const int k = lk[e];
  const uint64_t d = static_cast<uint64_t>(ldom[e]) << (bits + 1);
  if (k < np) {
    key[e] = d | static_cast<uint64_t>(k);
    atomicAdd(present + ldom[e], 1);
  } else {
    key[e] = d | (uint64_t{1} << bits) | static_cast<uint64_t>(gidx[k]);
  }
  val[e] = static_cast<int>(e);
}

// Every domain starts with all polynomial points, not inner unless the domain held them.
__global__ void merge_poly_kernel(Index n_slots, int np, const Index* __restrict__ gidx,
                                  const Index* __restrict__ foff, Index* __restrict__ pts,
                                  char* __restrict__ inner) {
  const Index x = thread_index();
  if (x >= n_slots) return;
  const Index d = x / np;
  const int k = static_cast<int>(x % np);
  pts[foff[d] + k] = gidx[k];
  inner[foff[d] + k] = 0;
}

__global__ void merge_write_kernel(const int* __restrict__ sval, Index m, const int* __restrict__ lk,
                                   const unsigned char* __restrict__ lin,
                                   const int* __restrict__ ldom, int np,
                                   const Index* __restrict__ gidx, const Index* __restrict__ leaf_off,
                                   const int* __restrict__ present, const Index* __restrict__ foff,
                                   Index* __restrict__ pts, char* __restrict__ inner) {
  const Index t = thread_index();
  if (t >= m) return;
  const int e = sval[t];
  const int d = ldom[e];
  const int k = lk[e];
  const Index pos = k < np ? foff[d] + k : foff[d] + np + (t - leaf_off[d] - present[d]);
  pts[pos] = gidx[k];
  inner[pos] = lin[e] ? 1 : 0;
}

// ---- coarse points ----------------------------------------------------------------------

struct ClusterSplit {
  Index begin, mid;
  int child[2];  // next-generation clusters of [begin, begin + mid) and the rest; -1 if empty
};

__global__ void coarse_init_kernel(Index m, int np, int* __restrict__ ck, int* __restrict__ ccl) {
  const Index t = thread_index();
  if (t >= m) return;
  ck[t] = np + static_cast<int>(t);
  ccl[t] = 0;
}

__global__ void cluster_apply_kernel(const int* __restrict__ perm, Index m, const int* __restrict__ ck,
                                     const int* __restrict__ ccl,
                                     const ClusterSplit* __restrict__ sp, int* __restrict__ ck2,
                                     int* __restrict__ ccl2) {
  const Index t = thread_index();
  if (t >= m) return;
  const int i = perm[t];
  const ClusterSplit& s = sp[ccl[i]];
  ck2[t] = ck[i];
  ccl2[t] = s.child[t - s.begin < s.mid ? 0 : 1];
}

// Squared distance to the cluster's bbox centre with the host's roundings
// (initialize_cluster, domain_divider.hpp:295-305).
__device__ __forceinline__ double centre_dist2(const double* __restrict__ x, Index n, int k,
                                               const double* __restrict__ ctr, int C, int c) {
  const double dx = __dsub_rn(x[k], ctr[c]);
  const double dy = __dsub_rn(x[n + k], ctr[C + c]);
  const double dz = __dsub_rn(x[2 * n + k], ctr[2 * static_cast<Index>(C) + c]);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// best[c] = smallest squared distance (as bits: non-negative doubles order as integers).
__global__ void centre_dist_kernel(const int* __restrict__ ck, const int* __restrict__ ccl, Index m,
                                   const double* __restrict__ x, Index n,
                                   const double* __restrict__ ctr, int C,
                                   unsigned long long* __restrict__ best) {
  const Index i = thread_index();
  if (i - static_cast<Index>(threadIdx.x & 31) >= m) return;
  const bool valid = i < m;
  const int c = valid ? ccl[i] : -1;
  const int c0 = __shfl_sync(kFull, c, 0);
  const bool uniform = __all_sync(kFull, !valid || c == c0);
  unsigned long long d =
      valid ? static_cast<unsigned long long>(__double_as_longlong(centre_dist2(x, n, ck[i], ctr, C, c)))
            : ~0ull;
  if (uniform) {
    for (int o = 16; o > 0; o >>= 1) d = min(d, __shfl_xor_sync(kFull, d, o));
    if ((threadIdx.x & 31) == 0) atomicMin(best + c0, d);
  } else if (valid) {
    atomicMin(best + c, d);
  }
}

// pos[c] = first position (in the cluster's order) at the smallest distance: ties go to the
// parent's lexicographic order, which is the order of the sorted segment.
__global__ void centre_pos_kernel(const int* __restrict__ ck, const int* __restrict__ ccl, Index m,
                                  const double* __restrict__ x, Index n,
                                  const double* __restrict__ ctr, int C,
                                  const unsigned long long* __restrict__ best,
                                  unsigned* __restrict__ pos) {
  const Index i = thread_index();
  if (i - static_cast<Index>(threadIdx.x & 31) >= m) return;
  const bool valid = i < m;
  const int c = valid ? ccl[i] : -1;
  const int c0 = __shfl_sync(kFull, c, 0);
  const bool uniform = __all_sync(kFull, !valid || c == c0);
  const bool hit =
      valid && static_cast<unsigned long long>(__double_as_longlong(centre_dist2(x, n, ck[i], ctr, C, c))) ==
                   best[c];
  const unsigned p = hit ? static_cast<unsigned>(i) : 0xffffffffu;
  if (uniform) {
    const unsigned q = __reduce_min_sync(kFull, p);
    if ((threadIdx.x & 31) == 0 && q != 0xffffffffu) atomicMin(pos + c0, q);
  } else if (hit) {
    atomicMin(pos + c, p);
  }
}

__global__ void centre_index_kernel(int C, const unsigned* __restrict__ pos, const int* __restrict__ ck,
                                    int* __restrict__ centre) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C) centre[c] = ck[pos[c]];
}

// Keys ordering clusters by volume, largest first (volumes are non-negative).
__global__ void volume_keys_kernel(int C, const double* __restrict__ vol, uint64_t* __restrict__ key,
                                   int* __restrict__ val) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  key[c] = ~static_cast<uint64_t>(__double_as_longlong(vol[c]));
  val[c] = c;
}

__global__ void mark_centres_kernel(int C, const int* __restrict__ centre,
                                    const unsigned char* __restrict__ use,
                                    unsigned char* __restrict__ sel) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C && (use == nullptr || use[c])) sel[centre[c]] = 1;
}

int bit_width(uint64_t v) { return static_cast<int>(std::bit_width(v)); }

}  // namespace

struct DeviceDivider::Impl {
  const double* coords;
  Index mu;
  std::vector<Index> poly;
  int np;
  Index n = 0;  // points of the current level
  DevBuf<Index> level;
  DevBuf<double> x, uq;
  DevBuf<unsigned> rank;
  int b = 1;  // bits of a rank
  DevBuf<uint64_t> k0, k1;
  DevBuf<int> v0, v1;
  DevBuf<unsigned char> tmp;

  void reserve_sort(Index m) {
    if (static_cast<Index>(k0.size()) >= m) return;
    k0.resize(m);
    k1.resize(m);
    v0.resize(m);
    v1.resize(m);
  }

  void radix(Index m, int end_bit) {
    size_t bytes = 0;
    PGPU_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, k0.data(), k1.data(), v0.data(),
                                              v1.data(), m, 0, end_bit, stream()));
    if (tmp.size() < bytes) tmp.resize(bytes);
    PGPU_CUDA(cub::DeviceRadixSort::SortPairs(tmp.data(), bytes, k0.data(), k1.data(), v0.data(),
                                              v1.data(), m, 0, end_bit, stream()));
  }

  // Orders the m elements by (segment, lexicographic rank key of the segment's axes); returns
  // the permutation (sorted position -> element).
  const int* segment_order(const int* el_k, const int* el_seg, Index m, int S,
                           const unsigned char* axes) {
    reserve_sort(m);
    minor_keys_kernel<<<blocks_for(m, 256), 256, 0, stream()>>>(el_k, el_seg, m, rank.data(), n,
                                                                axes, b, k0.data(), v0.data());
    PGPU_LAUNCH_CHECK();
    radix(m, 2 * b);
    major_keys_kernel<<<blocks_for(m, 256), 256, 0, stream()>>>(v1.data(), el_k, el_seg, m,
                                                                rank.data(), n, axes, b, k0.data(),
                                                                v0.data());
    PGPU_LAUNCH_CHECK();
    radix(m, bit_width(static_cast<uint64_t>(S - 1)) + b);
    return v1.data();
  }

  // Bbox of every segment: its axes, and optionally volume and centre.
  void segment_shape(const int* el_k, const int* el_seg, Index m, int S, DevBuf<unsigned char>& axes,
                     double* volume, double* ctr) {
    DevBuf<unsigned> mn(3 * static_cast<size_t>(S)), mx(3 * static_cast<size_t>(S));
    PGPU_CUDA(cudaMemsetAsync(mn.data(), 0xff, mn.size() * sizeof(unsigned), stream()));
    mx.zero();
    seg_bbox_kernel<<<blocks_for(m, 256), 256, 0, stream()>>>(el_k, el_seg, m, rank.data(), n, S,
                                                              mn.data(), mx.data());
    PGPU_LAUNCH_CHECK();
    axes.resize(S);
    seg_shape_kernel<<<blocks_for(S, 128), 128, 0, stream()>>>(S, mn.data(), mx.data(), uq.data(), n,
                                                               axes.data(), volume, ctr);
    PGPU_LAUNCH_CHECK();
  }
};

DeviceDivider::DeviceDivider(const double* coords, Index mu, const std::vector<Index>& poly)
    : impl_(new Impl) {
  impl_->coords = coords;
  impl_->mu = mu;
  impl_->poly = poly;
  impl_->np = static_cast<int>(poly.size());
}

DeviceDivider::~DeviceDivider() { delete impl_; }

void DeviceDivider::set_level(const std::vector<Index>& lv) {
  Impl& I = *impl_;
  const Index n = static_cast<Index>(lv.size());
  if (n >= (Index{1} << 31) - 1) throw_invalid("too many points for the device domain division");
  if (n < I.np) throw_runtime("level point list lacks the polynomial points");
  I.n = n;
  I.level.upload(lv);
  if (n == 0) return;
  I.x.resize(3 * n);
  gather_coords_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(I.coords, I.level.data(), n, I.x.data());
  PGPU_LAUNCH_CHECK();
  I.rank.resize(3 * n);
  I.uq.resize(3 * n);
  I.reserve_sort(n);
  DevBuf<unsigned> f(n), r(n);
  size_t sbytes = 0;
  PGPU_CUDA(cub::DeviceScan::InclusiveSum(nullptr, sbytes, f.data(), r.data(), n, stream()));
  DevBuf<unsigned char> stmp(sbytes);
  for (int a = 0; a < 3; ++a) {
    axis_keys_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(I.x.data() + a * n, n, I.k0.data(),
                                                               I.v0.data());
    PGPU_LAUNCH_CHECK();
    I.radix(n, 64);
    new_value_flags_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(I.k1.data(), n, f.data());
    PGPU_LAUNCH_CHECK();
    PGPU_CUDA(cub::DeviceScan::InclusiveSum(stmp.data(), sbytes, f.data(), r.data(), n, stream()));
    rank_scatter_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(r.data(), I.v1.data(),
                                                                  I.x.data() + a * n, n,
                                                                  I.rank.data() + a * n,
                                                                  I.uq.data() + a * n);
    PGPU_LAUNCH_CHECK();
  }
  I.b = std::max(1, bit_width(static_cast<uint64_t>(n - 1)));
}

void DeviceDivider::divide(LevelDomains& out) {
  Impl& I = *impl_;
  const Index n = I.n;
  const int np = I.np;

  // The plan: generation by generation, the domains that split (in the reference's list order)
  // and where each child goes: into the next generation or, at most 1024 points, out as a leaf.
  struct Gen {
    std::vector<DivSeg> segs;
    Index size = 0;
  };
  std::vector<Gen> gens;
  std::vector<Index> leaf_n, leaf_off;
  Index leaf_total = 0;
  {
    std::vector<Index> cur{n};
    int parent = -1;
    while (!cur.empty()) {
      Gen g;
      std::vector<Index> next;
      for (size_t j = 0; j < cur.size(); ++j) {
        const Index m = cur[j];
        DivSeg* ps = parent >= 0 ? &gens[parent].segs[j / 2] : nullptr;
        const int c = static_cast<int>(j % 2);
        if (m <= DomainDivider::kMaxLeafSize) {
          if (ps) {
            ps->dst[c] = leaf_total;
            ps->id[c] = static_cast<int>(leaf_n.size());
            ps->leaf[c] = 1;
          }
          leaf_off.push_back(leaf_total);
          leaf_n.push_back(m);
          leaf_total += m;
        } else {
          DivSeg s{};
          s.begin = g.size;
          s.n = m;
          overlap_split_sizes(m, s.left_part, s.mid, s.right_part);
          if (ps) {
            ps->dst[c] = g.size;
            ps->id[c] = static_cast<int>(g.segs.size());
            ps->leaf[c] = 0;
          }
          g.size += m;
          g.segs.push_back(s);
          next.push_back(s.right_part);
          next.push_back(m - s.left_part);
        }
      }
      gens.push_back(std::move(g));
      parent = static_cast<int>(gens.size()) - 1;
      cur = std::move(next);
    }
  }
  const Index n_dom = static_cast<Index>(leaf_n.size());
  if (leaf_total >= (Index{1} << 31) - 1) throw_invalid("too many points for the device domain division");

  DevBuf<int> lk(leaf_total), ldom(leaf_total);
  DevBuf<unsigned char> lin(leaf_total);
  Index max_gen = 0;
  for (const auto& g : gens) max_gen = std::max(max_gen, g.size);
  DevBuf<int> ek[2], eseg[2];
  DevBuf<unsigned char> ein[2];
  for (int h = 0; h < 2; ++h) {
    ek[h].resize(max_gen);
    eseg[h].resize(max_gen);
    ein[h].resize(max_gen);
  }
  if (gens[0].segs.empty()) {
    if (n > 0) {
      init_elements_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(n, lk.data(), lin.data(), ldom.data());
      PGPU_LAUNCH_CHECK();
    }
  } else {
    init_elements_kernel<<<blocks_for(n, 256), 256, 0, stream()>>>(n, ek[0].data(), ein[0].data(),
                                                                    eseg[0].data());
    PGPU_LAUNCH_CHECK();
  }
  int h = 0;
  for (size_t gi = 0; gi < gens.size() && !gens[gi].segs.empty(); ++gi) {
    const Gen& g = gens[gi];
    const int S = static_cast<int>(g.segs.size());
    const Index m = g.size;
    DevBuf<DivSeg> dsegs;
    dsegs.upload(g.segs);
    DevBuf<unsigned char> axes;
    I.segment_shape(ek[h].data(), eseg[h].data(), m, S, axes, nullptr, nullptr);
    const int* perm = I.segment_order(ek[h].data(), eseg[h].data(), m, S, axes.data());
    div_scatter_kernel<<<blocks_for(m, 256), 256, 0, stream()>>>(
        perm, m, ek[h].data(), ein[h].data(), eseg[h].data(), dsegs.data(), ek[1 - h].data(),
        ein[1 - h].data(), eseg[1 - h].data(), lk.data(), lin.data(), ldom.data());
    PGPU_LAUNCH_CHECK();
    h = 1 - h;
  }

  // Polynomial points first in every domain, the rest by ascending index.
  out.sizes.assign(n_dom, 0);
  DevBuf<int> present(std::max<Index>(n_dom, 1));
  present.zero();
  const int bits = std::max(4, bit_width(static_cast<uint64_t>(std::max<Index>(I.mu - 1, 1))));
  const int end_bit = bit_width(static_cast<uint64_t>(std::max<Index>(n_dom - 1, 0))) + bits + 1;
  if (end_bit > 64) throw_invalid("too many domains for the device domain division");
  if (leaf_total > 0) {
    I.reserve_sort(leaf_total);
    merge_keys_kernel<<<blocks_for(leaf_total, 256), 256, 0, stream()>>>(
        lk.data(), ldom.data(), leaf_total, np, I.level.data(), bits, I.k0.data(), I.v0.data(),
        present.data());
    PGPU_LAUNCH_CHECK();
    I.radix(leaf_total, end_bit);
  }
  std::vector<int> pres = present.to_host();
  std::vector<Index> foff(n_dom + 1, 0);
  for (Index d = 0; d < n_dom; ++d) {
    out.sizes[d] = leaf_n[d] - pres[d] + np;
    foff[d + 1] = foff[d] + out.sizes[d];
  }
  const Index total = foff[n_dom];
  out.pts.resize(total);
  out.inner.resize(total);
  if (total == 0) return;
  DevBuf<Index> dfoff, dleaf_off;
  dfoff.upload(foff);
  dleaf_off.upload(leaf_off);
  if (np > 0) {
    const Index slots = n_dom * np;
    merge_poly_kernel<<<blocks_for(slots, 256), 256, 0, stream()>>>(slots, np, I.level.data(), dfoff.data(),
                                                                    out.pts.data(), out.inner.data());
    PGPU_LAUNCH_CHECK();
  }
  if (leaf_total > 0) {
    merge_write_kernel<<<blocks_for(leaf_total, 256), 256, 0, stream()>>>(
        I.v1.data(), leaf_total, lk.data(), lin.data(), ldom.data(), np, I.level.data(),
        dleaf_off.data(), present.data(), dfoff.data(), out.pts.data(), out.inner.data());
    PGPU_LAUNCH_CHECK();
  }
}

std::vector<Index> DeviceDivider::choose_coarse_points(Index n_coarse) {
  Impl& I = *impl_;
  const Index n = I.n;
  const int np = I.np;
  const Index P = n - np;  // clustered points: the level's points after the polynomial ones
  std::vector<Index> result(I.poly);
  if (P <= 0) return result;

  struct Stats {
    DevBuf<unsigned char> axes;
    DevBuf<double> volume, ctr;
    DevBuf<unsigned long long> best;
    DevBuf<unsigned> pos;
    DevBuf<int> centre;
  };
  DevBuf<int> ck[2], ccl[2];
  for (int h = 0; h < 2; ++h) {
    ck[h].resize(P);
    ccl[h].resize(P);
  }
  coarse_init_kernel<<<blocks_for(P, 256), 256, 0, stream()>>>(P, np, ck[0].data(), ccl[0].data());
  PGPU_LAUNCH_CHECK();
  int h = 0;
  // Bbox, volume, centre and the point nearest to the centre of every cluster.
  auto stats = [&](int C, Stats& s) {
    s.volume.resize(C);
    s.ctr.resize(3 * static_cast<size_t>(C));
    I.segment_shape(ck[h].data(), ccl[h].data(), P, C, s.axes, s.volume.data(), s.ctr.data());
    s.best.resize(C);
    s.pos.resize(C);
    s.centre.resize(C);
    PGPU_CUDA(cudaMemsetAsync(s.best.data(), 0xff, C * sizeof(unsigned long long), stream()));
    PGPU_CUDA(cudaMemsetAsync(s.pos.data(), 0xff, C * sizeof(unsigned), stream()));
    centre_dist_kernel<<<blocks_for(P, 256), 256, 0, stream()>>>(ck[h].data(), ccl[h].data(), P,
                                                                 I.x.data(), n, s.ctr.data(), C,
                                                                 s.best.data());
    PGPU_LAUNCH_CHECK();
    centre_pos_kernel<<<blocks_for(P, 256), 256, 0, stream()>>>(ck[h].data(), ccl[h].data(), P,
                                                                I.x.data(), n, s.ctr.data(), C,
                                                                s.best.data(), s.pos.data());
    PGPU_LAUNCH_CHECK();
    centre_index_kernel<<<blocks_for(C, 256), 256, 0, stream()>>>(C, s.pos.data(), ck[h].data(),
                                                                  s.centre.data());
    PGPU_LAUNCH_CHECK();
  };
  DevBuf<unsigned char> sel(n);
  sel.zero();
  auto mark = [&](const Stats& s, int C, const std::vector<unsigned char>* use) {
    DevBuf<unsigned char> duse;
    if (use) duse.upload(*use);
    mark_centres_kernel<<<blocks_for(C, 256), 256, 0, stream()>>>(C, s.centre.data(),
                                                                  use ? duse.data() : nullptr, sel.data());
    PGPU_LAUNCH_CHECK();
  };

  Stats cur, nxt;
  std::vector<Index> sizes{P};  // cluster sizes in segment order
  stats(1, cur);
  Index count = 1;
  if (count >= n_coarse) mark(cur, 1, nullptr);
  while (count < n_coarse) {
    const int C = static_cast<int>(sizes.size());
    Index n_split = 0;
    for (Index s : sizes) n_split += s >= 2 ? 1 : 0;
    if (n_split == 0) {  // single-point clusters split into themselves
      mark(cur, C, nullptr);
      break;
    }
    // A generation whose splits cannot all be taken is the last one; its splits are accepted
    // in the reference's order (volume descending, domain_divider.hpp:65-70) until the count
    // is reached.
    const bool partial = count + n_split >= n_coarse;
    std::vector<ClusterSplit> sp(C);
    std::vector<Index> next;
    next.reserve(2 * sizes.size());
    Index begin = 0;
    for (int c = 0; c < C; ++c) {
      const Index mid = cluster_split(sizes[c]);
      sp[c] = ClusterSplit{begin, mid, {-1, -1}};
      if (mid > 0) {
        sp[c].child[0] = static_cast<int>(next.size());
        next.push_back(mid);
      }
      if (sizes[c] - mid > 0) {
        sp[c].child[1] = static_cast<int>(next.size());
        next.push_back(sizes[c] - mid);
      }
      begin += sizes[c];
    }
    DevBuf<ClusterSplit> dsp;
    dsp.upload(sp);
    const int* perm = I.segment_order(ck[h].data(), ccl[h].data(), P, C, cur.axes.data());
    cluster_apply_kernel<<<blocks_for(P, 256), 256, 0, stream()>>>(perm, P, ck[h].data(), ccl[h].data(),
                                                                   dsp.data(), ck[1 - h].data(),
                                                                   ccl[1 - h].data());
    PGPU_LAUNCH_CHECK();
    h = 1 - h;
    const int C2 = static_cast<int>(next.size());
    stats(C2, nxt);
    if (!partial) {
      count += n_split;
      sizes = std::move(next);
      std::swap(cur, nxt);
      continue;
    }
    volume_keys_kernel<<<blocks_for(C, 256), 256, 0, stream()>>>(C, cur.volume.data(), I.k0.data(),
                                                                 I.v0.data());
    PGPU_LAUNCH_CHECK();
    I.radix(C, 64);
    std::vector<int> order(C);
    PGPU_CUDA(cudaMemcpyAsync(order.data(), I.v1.data(), C * sizeof(int), cudaMemcpyDeviceToHost,
                              stream()));
    sync();
    std::vector<unsigned char> use_parent(C, 1), use_child(C2, 0);
    for (int t = 0; t < C && count < n_coarse; ++t) {
      const int c = order[t];
      use_parent[c] = 0;
      for (int ch : sp[c].child)
        if (ch >= 0) use_child[ch] = 1;
      count += sizes[c] >= 2 ? 1 : 0;
    }
    mark(cur, C, &use_parent);
    mark(nxt, C2, &use_child);
    break;
  }

  // The marked centres in level order, which is ascending index order after the polynomial
  // points.
  DevBuf<Index> picked(P);
  DevBuf<Index> n_picked(1);
  n_picked.zero();
  size_t bytes = 0;
  PGPU_CUDA(cub::DeviceSelect::Flagged(nullptr, bytes, I.level.data() + np, sel.data() + np,
                                       picked.data(), n_picked.data(), P, stream()));
  DevBuf<unsigned char> stmp(bytes);
  PGPU_CUDA(cub::DeviceSelect::Flagged(stmp.data(), bytes, I.level.data() + np, sel.data() + np,
                                       picked.data(), n_picked.data(), P, stream()));
  Index k = 0;
  PGPU_CUDA(cudaMemcpyAsync(&k, n_picked.data(), sizeof(Index), cudaMemcpyDeviceToHost, stream()));
  sync();
  result.resize(np + k);
  if (k > 0)
    PGPU_CUDA(cudaMemcpyAsync(result.data() + np, picked.data(), k * sizeof(Index),
                              cudaMemcpyDeviceToHost, stream()));
  sync();
  return result;
}

}  // namespace pgpu
