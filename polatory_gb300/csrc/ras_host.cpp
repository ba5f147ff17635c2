// Host-side RAS set-up: domain decomposition, coarse-point selection, unisolvent points.
// The splitting rules restate include/polatory/preconditioner/domain_divider.hpp:161-313; a
// selection (nth_element) replaces the full sort wherever only the partition into
// [0, k) / [k, n) of the sorted order matters, which yields the same point sets.
#include "ras_host.hpp"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>
#include <random>
#include <set>

namespace pgpu {

namespace {

struct MixedPoint {
  Index index;
  bool inner;
  bool grad;
  int mult() const { return grad ? 3 : 1; }
};

struct Geo {
  const double* pts;
  const double* gpts;
  const double* at(const MixedPoint& p) const {
    return p.grad ? gpts + 3 * p.index : pts + 3 * p.index;
  }
};

// Axes ordered by decreasing width (domain_divider.hpp:192-196).
std::array<int, 3> axes_by_width(const double* wmin, const double* wmax) {
  double width[3] = {wmax[0] - wmin[0], wmax[1] - wmin[1], wmax[2] - wmin[2]};
  std::array<int, 3> axes{0, 1, 2};
  std::sort(axes.begin(), axes.end(), [&](int i, int j) { return width[i] > width[j]; });
  return axes;
}

struct LexLess {
  const Geo* g;
  std::array<int, 3> axes;
  bool operator()(const MixedPoint& a, const MixedPoint& b) const {
    const double* p = g->at(a);
    const double* q = g->at(b);
    for (int ax : axes) {
      if (p[ax] != q[ax]) return p[ax] < q[ax];
    }
    return false;
  }
};

void bbox_of(const Geo& g, const std::vector<MixedPoint>& pts, double* mn, double* mx) {
  for (int k = 0; k < 3; ++k) {
    mn[k] = INFINITY;
    mx[k] = -INFINITY;
  }
  for (const auto& p : pts) {
    const double* c = g.at(p);
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], c[k]);
      mx[k] = std::max(mx[k], c[k]);
    }
  }
}

// ---- parallel selection for the large splits --------------------------------------------
// The first generations of a division split a few huge point sets, which one thread per set
// would do serially. Above this size a split runs data-parallel: the same point sets as
// nth_element at the same ranks (ties among identical points resolved arbitrarily, as
// nth_element does).
Index g_par_split_min = 262144;

// Bounding box of [b, e), parallel over the range.
void bbox_range_par(const Geo& g, const MixedPoint* pts, Index n, double* mn, double* mx) {
  for (int k = 0; k < 3; ++k) {
    mn[k] = INFINITY;
    mx[k] = -INFINITY;
  }
#pragma omp parallel
  {
    double lmn[3] = {INFINITY, INFINITY, INFINITY}, lmx[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma omp for schedule(static) nowait
    for (Index i = 0; i < n; ++i) {
      const double* c = g.at(pts[i]);
      for (int k = 0; k < 3; ++k) {
        lmn[k] = std::min(lmn[k], c[k]);
        lmx[k] = std::max(lmx[k], c[k]);
      }
    }
#pragma omp critical
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], lmn[k]);
      mx[k] = std::max(mx[k], lmx[k]);
    }
  }
}

// Rearranges pts[0, n) so that, for the sorted cut ranks c_0 < c_1 < ..., every slice
// [c_j, c_{j+1}) holds the elements of those ranks under less (what nth_element at each cut
// gives). Buckets by the primary coordinate (quantiles of a sample), counts in parallel, sorts
// only the buckets holding a cut, then scatters in parallel.
void par_multi_select(const Geo& g, MixedPoint* pts, Index n, const LexLess& less,
                      const std::vector<Index>& cuts) {
  const int ax0 = less.axes[0];
  // Primary keys gathered once (the points are scattered in memory).
  std::vector<double> keys(n);
#pragma omp parallel for schedule(static)
  for (Index i = 0; i < n; ++i) keys[i] = g.at(pts[i])[ax0];
  // Splitters: 4095 quantiles of a regular sample of the primary keys.
  const Index ns = std::min<Index>(n, 65536);
  std::vector<double> sample(ns);
  for (Index i = 0; i < ns; ++i) sample[i] = keys[(i * n) / ns];
  std::sort(sample.begin(), sample.end());
  std::vector<double> spl;
  const int nb_want = 4096;
  for (int j = 1; j < nb_want; ++j) {
    const double v = sample[(static_cast<Index>(j) * ns) / nb_want];
    if (spl.empty() || v > spl.back()) spl.push_back(v);
  }
  const int nb = static_cast<int>(spl.size()) + 1;
  auto bucket_of = [&](double k) {
    return static_cast<int>(std::upper_bound(spl.begin(), spl.end(), k) - spl.begin());
  };
  std::vector<int> bk(n);
  const int nt = omp_get_max_threads();
  std::vector<std::vector<Index>> cnt(nt, std::vector<Index>(nb, 0));
#pragma omp parallel
  {
    auto& c = cnt[omp_get_thread_num()];
#pragma omp for schedule(static)
    for (Index i = 0; i < n; ++i) {
      bk[i] = bucket_of(keys[i]);
      ++c[bk[i]];
    }
  }
  std::vector<Index> start(nb + 1, 0);
  for (int b = 0; b < nb; ++b) {
    Index t = 0;
    for (int th = 0; th < nt; ++th) t += cnt[th][b];
    start[b + 1] = start[b] + t;
  }
  // Group of an element: the number of cuts at or below its rank. Buckets without a cut
  // inside have one group for all their elements; the others are sorted and split exactly.
  std::vector<char> exact(nb, 0);
  for (Index c : cuts) {
    const int b = static_cast<int>(std::upper_bound(start.begin(), start.end(), c) - start.begin()) - 1;
    if (b >= 0 && b < nb && c > start[b]) exact[b] = 1;
  }
  auto group_of_rank = [&](Index r) {
    return static_cast<int>(std::upper_bound(cuts.begin(), cuts.end(), r) - cuts.begin());
  };
  std::vector<int> bucket_group(nb);
  for (int b = 0; b < nb; ++b) bucket_group[b] = group_of_rank(start[b]);
  // Elements of the exact buckets, sorted.
  std::vector<std::vector<MixedPoint>> ex(nb);
  for (Index i = 0; i < n; ++i)
    if (exact[bk[i]]) ex[bk[i]].push_back(pts[i]);
  std::vector<MixedPoint> out(n);
  const int ng = static_cast<int>(cuts.size()) + 1;
  std::vector<Index> gstart(ng + 1, 0);
  for (int j = 0; j < ng - 1; ++j) gstart[j + 1] = cuts[j];
  gstart[ng] = n;
  std::vector<Index> gfill(ng, 0);
  // Exact buckets first (sequential, they are small).
  for (int b = 0; b < nb; ++b) {
    if (!exact[b]) continue;
    auto& v = ex[b];
    std::sort(v.begin(), v.end(), less);
    for (Index j = 0; j < static_cast<Index>(v.size()); ++j) {
      const int gi = group_of_rank(start[b] + j);
      out[gstart[gi] + gfill[gi]++] = v[j];
    }
  }
  // The rest: per-thread counts per group, then a parallel scatter.
  std::vector<std::vector<Index>> gc(nt, std::vector<Index>(ng, 0));
#pragma omp parallel
  {
    auto& c = gc[omp_get_thread_num()];
#pragma omp for schedule(static)
    for (Index i = 0; i < n; ++i)
      if (!exact[bk[i]]) ++c[bucket_group[bk[i]]];
  }
  std::vector<std::vector<Index>> goff(nt, std::vector<Index>(ng, 0));
  for (int gi = 0; gi < ng; ++gi) {
    Index o = gstart[gi] + gfill[gi];
    for (int th = 0; th < nt; ++th) {
      goff[th][gi] = o;
      o += gc[th][gi];
    }
  }
#pragma omp parallel
  {
    auto& o = goff[omp_get_thread_num()];
#pragma omp for schedule(static)
    for (Index i = 0; i < n; ++i)
      if (!exact[bk[i]]) out[o[bucket_group[bk[i]]]++] = pts[i];
  }
#pragma omp parallel for schedule(static)
  for (Index i = 0; i < n; ++i) pts[i] = out[i];
}

// std::ceil((d - 0.5) / 2.0) + std::floor((d + 0.5) / 2.0) (domain_divider.hpp:311-313).
double round_half_to_even(double d) { return std::ceil((d - 0.5) / 2.0) + std::floor((d + 0.5) / 2.0); }

// Index of the last prefix-sum entry <= v (upper_bound - 1).
Index last_le(const std::vector<Index>& prefix, Index v) {
  return static_cast<Index>(std::upper_bound(prefix.begin(), prefix.end(), v) - prefix.begin()) - 1;
}

// Splits one domain into two overlapping halves (domain_divider.hpp:161-269).
void divide_domain(const Geo& g, const Domain& d, Domain& left, Domain& right, bool par_ok) {
  const Index mu = d.num_points(), sigma = d.num_grad_points();
  const bool par = par_ok && sigma == 0 && mu >= g_par_split_min;
  std::vector<MixedPoint> mp(mu + sigma);
#pragma omp parallel for schedule(static) if (par)
  for (Index i = 0; i < mu; ++i) mp[i] = {d.point_indices[i], d.inner_point[i] != 0, false};
  for (Index i = 0; i < sigma; ++i)
    mp[mu + i] = {d.grad_point_indices[i], d.inner_grad_point[i] != 0, true};

  double mn[3], mx[3];
  if (par) bbox_range_par(g, mp.data(), static_cast<Index>(mp.size()), mn, mx);
  else bbox_of(g, mp, mn, mx);
  LexLess less{&g, axes_by_width(mn, mx)};

  const Index n_points = mu + sigma;
  const Index n_mult = mu + 3 * sigma;
  Index left_mult, mid_mult, right_mult;
  overlap_split_sizes(n_mult, left_mult, mid_mult, right_mult);

  Index left_part, right_part, mid;
  if (sigma == 0) {
    // Multiplicities are all one: the partition points are the multiplicity targets.
    left_part = left_mult;
    right_part = right_mult;
    mid = mid_mult;
    if (par) {
      std::vector<Index> cuts;
      for (Index c : {left_part, mid, right_part})
        if (c > 0 && c < n_points && (cuts.empty() || c > cuts.back())) cuts.push_back(c);
      par_multi_select(g, mp.data(), n_points, less, cuts);
    } else {
      std::nth_element(mp.begin(), mp.begin() + mid, mp.end(), less);
      if (left_part < mid) std::nth_element(mp.begin(), mp.begin() + left_part, mp.begin() + mid, less);
      if (right_part > mid && right_part < n_points)
        std::nth_element(mp.begin() + mid, mp.begin() + right_part, mp.end(), less);
    }
  } else {
    std::sort(mp.begin(), mp.end(), less);
    std::vector<Index> prefix{0};
    prefix.reserve(n_points + 1);
    for (const auto& p : mp) prefix.push_back(prefix.back() + p.mult());
    left_part = last_le(prefix, left_mult);
    right_part = last_le(prefix, right_mult);
    mid = last_le(prefix, mid_mult);
  }

  if (par) {
    // Value points only: fill both halves in parallel.
    left.point_indices.resize(right_part);
    left.inner_point.resize(right_part);
    right.point_indices.resize(n_points - left_part);
    right.inner_point.resize(n_points - left_part);
#pragma omp parallel for schedule(static)
    for (Index i = 0; i < n_points; ++i) {
      const auto& p = mp[i];
      if (i < right_part) {
        left.point_indices[i] = p.index;
        left.inner_point[i] = (p.inner && i < mid) ? 1 : 0;
      }
      if (i >= left_part) {
        right.point_indices[i - left_part] = p.index;
        right.inner_point[i - left_part] = (p.inner && i >= mid) ? 1 : 0;
      }
    }
    return;
  }
  for (Index i = 0; i < right_part; ++i) {
    const auto& p = mp[i];
    const char inner = (p.inner && i < mid) ? 1 : 0;
    if (p.grad) {
      left.grad_point_indices.push_back(p.index);
      left.inner_grad_point.push_back(inner);
    } else {
      left.point_indices.push_back(p.index);
      left.inner_point.push_back(inner);
    }
  }
  for (Index i = left_part; i < n_points; ++i) {
    const auto& p = mp[i];
    const char inner = (p.inner && i >= mid) ? 1 : 0;
    if (p.grad) {
      right.grad_point_indices.push_back(p.index);
      right.inner_grad_point.push_back(inner);
    } else {
      right.point_indices.push_back(p.index);
      right.inner_point.push_back(inner);
    }
  }
}

// Domain::merge_poly_points (domain.hpp:27-49): sort by index, put the polynomial points
// first (inner only where the domain already owned them).
void merge_poly_points(Domain& d, const std::vector<Index>& poly) {
  std::vector<std::pair<Index, char>> z(d.point_indices.size());
  for (size_t i = 0; i < z.size(); ++i) z[i] = {d.point_indices[i], d.inner_point[i]};
  std::sort(z.begin(), z.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  const Index np = static_cast<Index>(poly.size());
  std::vector<char> poly_inner(np, 0);
  std::vector<char> erase(z.size(), 0);
  for (Index i = 0; i < np; ++i) {
    auto it = std::lower_bound(z.begin(), z.end(), poly[i],
                               [](const auto& a, Index v) { return a.first < v; });
    if (it == z.end() || it->first != poly[i]) continue;
    poly_inner[i] = it->second;
    erase[it - z.begin()] = 1;
  }
  d.point_indices.clear();
  d.inner_point.clear();
  for (Index i = 0; i < np; ++i) {
    d.point_indices.push_back(poly[i]);
    d.inner_point.push_back(poly_inner[i]);
  }
  for (size_t i = 0; i < z.size(); ++i) {
    if (erase[i]) continue;
    d.point_indices.push_back(z[i].first);
    d.inner_point.push_back(z[i].second);
  }
}

// A cluster of the coarse-point selection: a segment [b, e) of one shared point array.
struct Segment {
  Index b = 0, e = 0;
  double volume = 0;
  MixedPoint center{};
  bool has_grad = false;
};

// initialize_cluster (domain_divider.hpp:277-308): bbox volume, the point nearest to the bbox
// centre, and (for clusters holding gradient points) the lexicographic sort used by the next
// split; value-only clusters are partitioned with nth_element at split time instead.
// parent_less: the parent's lexicographic order, which decides ties in the distance to the
// bbox centre (the reference takes the first such point in its sorted parent order; two-point
// clusters always tie). nullptr for the root (input order).
void init_segment(const Geo& g, std::vector<MixedPoint>& pts, Segment& s,
                  const LexLess* parent_less = nullptr, bool par = false) {
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  s.has_grad = false;
  if (par) {
    bbox_range_par(g, pts.data() + s.b, s.e - s.b, mn, mx);
    for (Index i = s.b; i < s.e && !s.has_grad; ++i) s.has_grad |= pts[i].grad;
  } else {
    for (Index i = s.b; i < s.e; ++i) {
      const double* c = g.at(pts[i]);
      for (int k = 0; k < 3; ++k) {
        mn[k] = std::min(mn[k], c[k]);
        mx[k] = std::max(mx[k], c[k]);
      }
      s.has_grad |= pts[i].grad;
    }
  }
  s.volume = (mx[0] - mn[0]) * (mx[1] - mn[1]) * (mx[2] - mn[2]);
  double ctr[3];
  for (int k = 0; k < 3; ++k) ctr[k] = mn[k] + (mx[k] - mn[k]) / 2.0;
  // The point nearest to the centre; ties go to the parent's lexicographic order, then to the
  // earlier position (chunks are combined in order, so the parallel scan picks the same one).
  auto better = [&](double d2, const MixedPoint& p, double best, const MixedPoint& cur) {
    return d2 < best || (d2 == best && parent_less && (*parent_less)(p, cur));
  };
  auto scan = [&](Index b, Index e, double& best, MixedPoint& c) {
    for (Index i = b; i < e; ++i) {
      const double* q = g.at(pts[i]);
      double dx = q[0] - ctr[0], dy = q[1] - ctr[1], dz = q[2] - ctr[2];
      double d2 = dx * dx + dy * dy + dz * dz;
      if (better(d2, pts[i], best, c)) {
        best = d2;
        c = pts[i];
      }
    }
  };
  double best = INFINITY;
  if (par) {
    const int nt = omp_get_max_threads();
    std::vector<double> tb(nt, INFINITY);
    std::vector<MixedPoint> tc(nt, s.center);
    const Index n = s.e - s.b;
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num();
      const Index b = s.b + (n * t) / nt, e = s.b + (n * (t + 1)) / nt;
      scan(b, e, tb[t], tc[t]);
    }
    for (int t = 0; t < nt; ++t)
      if (tb[t] < INFINITY && better(tb[t], tc[t], best, s.center)) {
        best = tb[t];
        s.center = tc[t];
      }
  } else {
    scan(s.b, s.e, best, s.center);
  }
  if (s.has_grad) {
    LexLess less{&g, axes_by_width(mn, mx)};
    std::sort(pts.begin() + s.b, pts.begin() + s.e, less);
  }
}

// Splits a segment at the position minimising |2 prefix(i) - size| with the tie rule of
// std::min_element and the comparator of domain_divider.hpp:82-88; children are initialised.
void split_segment(const Geo& g, std::vector<MixedPoint>& pts, const Segment& s, Segment& left,
                   Segment& right, bool par_ok = false) {
  const Index n = s.e - s.b;
  const bool par = par_ok && !s.has_grad && n >= g_par_split_min;
  Index mid = 0;
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  if (par) {
    bbox_range_par(g, pts.data() + s.b, n, mn, mx);
  } else {
    for (Index i = s.b; i < s.e; ++i) {
      const double* c = g.at(pts[i]);
      for (int k = 0; k < 3; ++k) {
        mn[k] = std::min(mn[k], c[k]);
        mx[k] = std::max(mx[k], c[k]);
      }
    }
  }
  const LexLess less{&g, axes_by_width(mn, mx)};
  if (s.has_grad) {
    std::vector<Index> prefix{0};
    prefix.reserve(n + 1);
    for (Index i = s.b; i < s.e; ++i) prefix.push_back(prefix.back() + pts[i].mult());
    const Index size = prefix.back();
    Index bestd = std::llabs(2 * prefix[0] - size);
    for (Index i = 1; i < n; ++i) {
      Index di = std::llabs(2 * prefix[i] - size);
      if (di < bestd || (di == bestd && i % 2 == 0)) {
        mid = i;
        bestd = di;
      }
    }
  } else {
    mid = cluster_split(n);
    if (mid > 0 && mid < n) {
      if (par)
        par_multi_select(g, pts.data() + s.b, n, less, {mid});
      else
        std::nth_element(pts.begin() + s.b, pts.begin() + s.b + mid, pts.begin() + s.e, less);
    }
  }
  left.b = s.b;
  left.e = s.b + mid;
  right.b = s.b + mid;
  right.e = s.e;
  if (left.e > left.b) init_segment(g, pts, left, &less, par);
  if (right.e > right.b) init_segment(g, pts, right, &less, par);
}

}  // namespace

void set_parallel_split_min(Index n) { g_par_split_min = n; }

void overlap_split_sizes(Index n, Index& left_part, Index& mid, Index& right_part) {
  const double q = DomainDivider::kOverlapQuota * 1024.0 / static_cast<double>(n);
  const Index n_sub = static_cast<Index>(round_half_to_even((1.0 + q) / 2.0 * static_cast<double>(n)));
  left_part = n - n_sub;
  right_part = n_sub;
  mid = static_cast<Index>(round_half_to_even(static_cast<double>(left_part + right_part) / 2.0));
}

// The first i in [1, n) minimising |2 i - n|, a tie going to the even i (std::min_element over
// domain_divider.hpp:82-88's comparator); 0 for n < 2. For odd n both neighbours of n / 2 tie.
Index cluster_split(Index n) {
  if (n < 2) return 0;
  if (n % 2 == 0) return n / 2;
  const Index a = (n - 1) / 2;
  return a % 2 == 0 ? a : a + 1;
}

DomainDivider::DomainDivider(const double* points, const double* grad_points,
                             const std::vector<Index>& point_indices,
                             const std::vector<Index>& grad_point_indices,
                             const std::vector<Index>& poly_point_indices)
    : points_(points),
      grad_points_(grad_points),
      point_idcs_(point_indices),
      grad_point_idcs_(grad_point_indices),
      poly_point_idcs_(poly_point_indices) {
  Geo g{points_, grad_points_};
  Domain root;
  root.point_indices = point_indices;
  root.grad_point_indices = grad_point_indices;
  root.inner_point.assign(point_indices.size(), 1);
  root.inner_grad_point.assign(grad_point_indices.size(), 1);

  // Breadth-first: every generation is split in parallel; leaves are kept in order.
  std::vector<Domain> current;
  current.push_back(std::move(root));
  while (!current.empty()) {
    const Index n = static_cast<Index>(current.size());
    std::vector<char> split(n, 0);
    std::vector<Domain> lefts(n), rights(n);
    std::vector<Index> big, small;
    Index n_split = 0;
    for (Index i = 0; i < n; ++i) {
      const auto& d = current[i];
      if (d.num_points() + 3 * d.num_grad_points() > kMaxLeafSize) ++n_split;
    }
    // While there are fewer domains to split than threads, the huge ones split data-parallel.
    const bool few = n_split < omp_get_max_threads();
    for (Index i = 0; i < n; ++i) {
      const auto& d = current[i];
      if (d.num_points() + 3 * d.num_grad_points() <= kMaxLeafSize) continue;
      split[i] = 1;
      (few && d.num_grad_points() == 0 && d.num_points() >= g_par_split_min ? big : small).push_back(i);
    }
    // Huge domains one at a time, each split data-parallel; the rest one per thread.
    for (Index i : big) divide_domain(g, current[i], lefts[i], rights[i], true);
    const Index ns = static_cast<Index>(small.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (Index k = 0; k < ns; ++k)
      divide_domain(g, current[small[k]], lefts[small[k]], rights[small[k]], false);
    std::vector<Domain> next;
    for (Index i = 0; i < n; ++i) {
      if (!split[i]) {
        domains_.push_back(std::move(current[i]));
      } else {
        next.push_back(std::move(lefts[i]));
        next.push_back(std::move(rights[i]));
      }
    }
    current = std::move(next);
  }
  const Index nd = static_cast<Index>(domains_.size());
#pragma omp parallel for schedule(dynamic, 16)
  for (Index i = 0; i < nd; ++i) merge_poly_points(domains_[i], poly_point_idcs_);
}

std::pair<std::vector<Index>, std::vector<Index>> DomainDivider::choose_coarse_points(
    Index n_coarse) const {
  return choose_coarse_points(points_, grad_points_, point_idcs_, grad_point_idcs_,
                              poly_point_idcs_, n_coarse);
}

std::pair<std::vector<Index>, std::vector<Index>> DomainDivider::choose_coarse_points(
    const double* points_, const double* grad_points_, const std::vector<Index>& point_idcs_,
    const std::vector<Index>& grad_point_idcs_, const std::vector<Index>& poly_point_idcs_,
    Index n_coarse) {
  // The reference pops clusters from a priority queue ordered by (level ascending, bbox volume
  // descending), splits each at its median and keeps the centres (domain_divider.hpp:54-125).
  // That order visits the clusters level by level, so here every level is split at once, in
  // place on one point array and in parallel; the splits are then accepted in the reference's
  // order (volume descending) until the centre count reaches n_coarse, and the remaining
  // clusters of that level stay whole. Apart from ties in volume this yields the same sets.
  Geo g{points_, grad_points_};
  std::vector<Index> idcs(poly_point_idcs_);
  std::vector<Index> grad_idcs;

  std::vector<char> is_poly;
  {
    Index maxi = 0;
    for (auto i : point_idcs_) maxi = std::max(maxi, i);
    is_poly.assign(maxi + 1, 0);
    for (auto i : poly_point_idcs_)
      if (i <= maxi) is_poly[i] = 1;
  }
  std::vector<MixedPoint> pts;
  pts.reserve(point_idcs_.size() + grad_point_idcs_.size());
  for (auto i : point_idcs_)
    if (!is_poly[i]) pts.push_back({i, true, false});
  for (auto i : grad_point_idcs_) pts.push_back({i, true, true});

  std::vector<Segment> cur(1);
  cur[0].b = 0;
  cur[0].e = static_cast<Index>(pts.size());
  std::vector<Segment> finals;
  if (pts.empty()) return {std::move(idcs), std::move(grad_idcs)};
  init_segment(g, pts, cur[0], nullptr, static_cast<Index>(pts.size()) >= g_par_split_min);
  Index count = cur[0].center.mult();

  while (count < n_coarse && !cur.empty()) {
    const Index ns = static_cast<Index>(cur.size());
    // Single-point clusters split into themselves: stop when no cluster can grow the count.
    if (std::none_of(cur.begin(), cur.end(), [](const Segment& c) { return c.e - c.b >= 2; })) break;
    std::vector<Segment> left(ns), right(ns);
    if (ns < omp_get_max_threads()) {
      // Few clusters: split them one at a time, each data-parallel when huge.
      for (Index s = 0; s < ns; ++s) split_segment(g, pts, cur[s], left[s], right[s], true);
    } else {
#pragma omp parallel for schedule(dynamic, 1)
      for (Index s = 0; s < ns; ++s) split_segment(g, pts, cur[s], left[s], right[s]);
    }
    // Accept the splits in the reference's order (volume descending); clusters of equal volume
    // in the order of their segments.
    std::vector<Index> order(ns);
    for (Index s = 0; s < ns; ++s) order[s] = s;
    std::sort(order.begin(), order.end(), [&](Index a, Index b) {
      if (cur[a].volume != cur[b].volume) return cur[a].volume > cur[b].volume;
      return cur[a].b < cur[b].b;
    });
    std::vector<Segment> next;
    next.reserve(2 * ns);
    Index k = 0;
    for (; k < ns && count < n_coarse; ++k) {
      const Index s = order[k];
      count -= cur[s].center.mult();
      for (Segment* c : {&left[s], &right[s]}) {
        if (c->e > c->b) {
          count += c->center.mult();
          next.push_back(*c);
        }
      }
    }
    for (; k < ns; ++k) finals.push_back(cur[order[k]]);
    cur = std::move(next);
  }
  // The centres in ascending index order after the polynomial points: a canonical order that
  // does not depend on how the clusters were visited.
  std::vector<Index> centers;
  for (const auto* v : {&finals, &cur})
    for (const auto& s : *v) (s.center.grad ? grad_idcs : centers).push_back(s.center.index);
  std::sort(centers.begin(), centers.end());
  std::sort(grad_idcs.begin(), grad_idcs.end());
  idcs.insert(idcs.end(), centers.begin(), centers.end());
  return {std::move(idcs), std::move(grad_idcs)};
}

void monomial_row(int degree, const double* p, double* out) {
  out[0] = 1.0;
  if (degree >= 1) {
    out[1] = p[0];
    out[2] = p[1];
    out[3] = p[2];
  }
  if (degree >= 2) {
    out[4] = p[0] * p[0];
    out[5] = p[0] * p[1];
    out[6] = p[0] * p[2];
    out[7] = p[1] * p[1];
    out[8] = p[1] * p[2];
    out[9] = p[2] * p[2];
  }
}

namespace {

// Full-pivoting LU inverse with Eigen's default rank threshold (epsilon * size * max pivot).
// Returns false when the matrix is rank deficient.
bool full_piv_inverse(std::vector<double> a, int n, std::vector<double>& inv) {
  std::vector<int> rp(n), cp(n);
  std::iota(rp.begin(), rp.end(), 0);
  std::iota(cp.begin(), cp.end(), 0);
  double max_pivot = 0;
  int rank = 0;
  for (int k = 0; k < n; ++k) {
    int bi = k, bj = k;
    double best = -1;
    for (int i = k; i < n; ++i)
      for (int j = k; j < n; ++j) {
        double v = std::fabs(a[i * n + j]);
        if (v > best) {
          best = v;
          bi = i;
          bj = j;
        }
      }
    if (k == 0) max_pivot = best;
    if (bi != k) {
      for (int j = 0; j < n; ++j) std::swap(a[k * n + j], a[bi * n + j]);
      std::swap(rp[k], rp[bi]);
    }
    if (bj != k) {
      for (int i = 0; i < n; ++i) std::swap(a[i * n + k], a[i * n + bj]);
      std::swap(cp[k], cp[bj]);
    }
    double piv = a[k * n + k];
    if (std::fabs(piv) > std::numeric_limits<double>::epsilon() * n * max_pivot) ++rank;
    if (piv == 0.0) continue;
    for (int i = k + 1; i < n; ++i) {
      double f = a[i * n + k] / piv;
      a[i * n + k] = f;
      for (int j = k + 1; j < n; ++j) a[i * n + j] -= f * a[k * n + j];
    }
  }
  if (rank < n) return false;
  // Solve for each unit vector: P A Q = L U  =>  A^{-1} = Q U^{-1} L^{-1} P.
  inv.assign(n * n, 0.0);
  std::vector<double> x(n);
  for (int c = 0; c < n; ++c) {
    for (int i = 0; i < n; ++i) x[i] = (rp[i] == c) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) x[i] -= a[i * n + j] * x[j];
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) x[i] -= a[i * n + j] * x[j];
      x[i] /= a[i * n + i];
    }
    for (int i = 0; i < n; ++i) inv[cp[i] * n + c] = x[i];
  }
  return true;
}

double l1_norm(const std::vector<double>& a, int n) {
  double best = 0;
  for (int j = 0; j < n; ++j) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += std::fabs(a[i * n + j]);
    best = std::max(best, s);
  }
  return best;
}

}  // namespace

std::vector<double> lagrange_coeffs(int degree, const double* poly_points, Index l,
                                    double* rcond_out) {
  const int n = static_cast<int>(l);
  std::vector<double> p(n * n);
  for (int i = 0; i < n; ++i) monomial_row(degree, poly_points + 3 * i, p.data() + i * n);
  std::vector<double> inv;
  if (!full_piv_inverse(p, n, inv)) throw_invalid("the set of points is not unisolvent");
  if (rcond_out) *rcond_out = 1.0 / (l1_norm(p, n) * l1_norm(inv, n));
  return inv;
}

std::vector<double> lagrange_coeffs_of(const std::vector<double>& rows, Index l) {
  std::vector<double> inv;
  if (!full_piv_inverse(rows, static_cast<int>(l), inv))
    throw_invalid("the set of points is not unisolvent");
  return inv;
}

std::vector<Index> unisolvent_point_set(const double* points, Index n, int degree) {
  std::vector<Index> out;
  if (degree < 0) return out;
  const int l = (degree + 1) * (degree + 2) * (degree + 3) / 6;
  std::mt19937 gen;
  std::uniform_int_distribution<Index> dist(Index{0}, n - 1);
  std::set<Index> best_set;
  double best_rcond = 0.0;
  bool found = false;
  for (int trial = 0; trial < 100; ++trial) {
    std::set<Index> set;
    while (static_cast<Index>(set.size()) < l) set.insert(dist(gen));
    std::vector<double> pp;
    for (auto i : set)
      for (int k = 0; k < 3; ++k) pp.push_back(points[3 * i + k]);
    try {
      double rc = 0;
      lagrange_coeffs(degree, pp.data(), l, &rc);
      if (best_rcond < rc) {
        best_rcond = rc;
        best_set = std::move(set);
      }
      found = true;
    } catch (const Error&) {
    }
  }
  if (!found) throw_runtime("could not find a unisolvent set of points");
  out.assign(best_set.begin(), best_set.end());
  return out;
}

}  // namespace pgpu
