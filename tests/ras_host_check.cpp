// CPU checks of the RAS host set-up (compiled and run by tests/test_ras_host.py):
//  1. the invariants of the reference's test/preconditioner/test_domain_divider.cpp:18-90
//     (inner points partition the level, polynomial points lead every domain, no duplicates,
//     coarse-point count within [n + l, n + l + 3));
//  2. domain sizes (points + 3 x gradient points) at most 1024;
//  3. the level-parallel coarse-point selection returns the same set as a direct sequential
//     restatement of the priority-queue rule (domain_divider.hpp:54-125) on value points, in
//     the canonical order (polynomial points, then ascending index);
//  4. asking for more coarse points than there are points returns every point once;
//  5. the Lagrange basis of test/polynomial/test_lagrange_basis.cpp:16-31: at a unisolvent
//     point set (degrees 0-2) the basis evaluates to the identity (to 1e-12), also for the
//     one-point-plus-one-gradient-point set of degree 1 (lagrange_basis.hpp:36-37), and a
//     repeated point set is rejected as not unisolvent.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <queue>
#include <random>
#include <set>
#include <vector>

#include "ras_host.hpp"

using pgpu::Index;

static int failures = 0;
#define CHECK(c)                                                          \
  do {                                                                    \
    if (!(c)) {                                                           \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);          \
      ++failures;                                                         \
    }                                                                     \
  } while (0)

static void check_divider(Index n_points, Index n_grad, Index n_poly, unsigned seed) {
  std::mt19937 gen(seed);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::vector<double> pts(3 * n_points), gpts(3 * std::max<Index>(n_grad, 1));
  for (auto& v : pts) v = u(gen);
  for (auto& v : gpts) v = u(gen);
  std::vector<Index> idx(n_points), gidx(n_grad);
  std::iota(idx.begin(), idx.end(), 0);
  std::iota(gidx.begin(), gidx.end(), 0);
  std::vector<Index> poly(idx.begin(), idx.begin() + n_poly);
  pgpu::DomainDivider div(pts.data(), gpts.data(), idx, gidx, poly);
  std::vector<Index> inner, ginner;
  for (const auto& d : div.domains()) {
    for (Index i = 0; i < d.num_points(); ++i)
      if (d.inner_point[i]) inner.push_back(d.point_indices[i]);
    for (Index i = 0; i < d.num_grad_points(); ++i)
      if (d.inner_grad_point[i]) ginner.push_back(d.grad_point_indices[i]);
    for (Index i = 0; i < n_poly; ++i) CHECK(d.point_indices[i] == poly[i]);
    auto a = d.point_indices;
    std::sort(a.begin(), a.end());
    CHECK(std::unique(a.begin(), a.end()) == a.end());
    auto b = d.grad_point_indices;
    std::sort(b.begin(), b.end());
    CHECK(std::unique(b.begin(), b.end()) == b.end());
    CHECK(d.num_points() - n_poly + 3 * d.num_grad_points() <= 1024 + n_poly);
  }
  CHECK(static_cast<Index>(inner.size()) == n_points);
  CHECK(static_cast<Index>(ginner.size()) == n_grad);
  std::sort(inner.begin(), inner.end());
  CHECK(std::unique(inner.begin(), inner.end()) == inner.end());
  std::sort(ginner.begin(), ginner.end());
  CHECK(std::unique(ginner.begin(), ginner.end()) == ginner.end());

  const Index n_coarse = 1000;
  auto [cp, cgp] = div.choose_coarse_points(n_coarse);
  const Index total = static_cast<Index>(cp.size()) + 3 * static_cast<Index>(cgp.size());
  CHECK(n_coarse + n_poly <= total);
  // The reference's bound is n + l + 3; a last split that replaces a value centre by two
  // gradient centres adds 5, so the loop can stop at most 4 above n + l.
  CHECK(total < n_coarse + n_poly + 5);
  for (Index i = 0; i < n_poly; ++i) CHECK(cp[i] == poly[i]);
}

// Sequential restatement of the priority-queue selection for value points only.
struct Cl {
  int level;
  double volume;
  std::vector<Index> pts;
  Index center;
};

static void init_cl(const std::vector<double>& p, Cl& c) {
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (Index i : c.pts)
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], p[3 * i + k]);
      mx[k] = std::max(mx[k], p[3 * i + k]);
    }
  c.volume = (mx[0] - mn[0]) * (mx[1] - mn[1]) * (mx[2] - mn[2]);
  double best = INFINITY;
  for (Index i : c.pts) {
    double d2 = 0;
    for (int k = 0; k < 3; ++k) {
      double dd = p[3 * i + k] - (mn[k] + (mx[k] - mn[k]) / 2.0);
      d2 += dd * dd;
    }
    if (d2 < best) {
      best = d2;
      c.center = i;
    }
  }
  double w[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  int axes[3] = {0, 1, 2};
  std::sort(axes, axes + 3, [&](int a, int b) { return w[a] > w[b]; });
  std::sort(c.pts.begin(), c.pts.end(), [&](Index a, Index b) {
    for (int ax : axes)
      if (p[3 * a + ax] != p[3 * b + ax]) return p[3 * a + ax] < p[3 * b + ax];
    return false;
  });
}

static void check_coarse_equivalence(Index n, Index n_coarse, unsigned seed) {
  std::mt19937 gen(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::vector<double> p(3 * n);
  for (auto& v : p) v = u(gen);
  std::vector<Index> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::vector<Index> poly{0, 1, 2, 3};
  std::vector<Index> none;
  pgpu::DomainDivider div(p.data(), nullptr, idx, none, poly);
  auto got = div.choose_coarse_points(n_coarse).first;

  auto cmp = [](const Cl* a, const Cl* b) {
    if (a->level != b->level) return a->level > b->level;
    return a->volume < b->volume;
  };
  std::priority_queue<Cl*, std::vector<Cl*>, decltype(cmp)> pq(cmp);
  auto* root = new Cl{0, 0, {}, 0};
  for (Index i = 4; i < n; ++i) root->pts.push_back(i);
  init_cl(p, *root);
  Index count = 1;
  pq.push(root);
  while (count < n_coarse) {
    Cl* c = pq.top();
    const Index m = static_cast<Index>(c->pts.size());
    Index mid = 0, bestd = m;
    for (Index i = 1; i < m; ++i) {
      Index di = std::llabs(2 * i - m);
      if (di < bestd || (di == bestd && i % 2 == 0)) {
        mid = i;
        bestd = di;
      }
    }
    pq.pop();
    --count;
    std::vector<Index> l(c->pts.begin(), c->pts.begin() + mid), r(c->pts.begin() + mid, c->pts.end());
    for (auto* v : {&l, &r}) {
      if (v->empty()) continue;
      auto* ch = new Cl{c->level + 1, 0, std::move(*v), 0};
      init_cl(p, *ch);
      ++count;
      pq.push(ch);
    }
    delete c;
  }
  std::vector<Index> want(poly);
  while (!pq.empty()) {
    want.push_back(pq.top()->center);
    delete pq.top();
    pq.pop();
  }
  std::set<Index> a(got.begin(), got.end()), b(want.begin(), want.end());
  CHECK(a == b);
  CHECK(got.size() == want.size());
  CHECK(std::equal(poly.begin(), poly.end(), got.begin()));
  CHECK(std::is_sorted(got.begin() + static_cast<std::ptrdiff_t>(poly.size()), got.end()));
}

// Single-point clusters split into themselves, so the selection stops when every cluster is a
// single point, with every point a centre.
static void check_coarse_saturation(Index n, unsigned seed) {
  std::mt19937 gen(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::vector<double> p(3 * n);
  for (auto& v : p) v = u(gen);
  std::vector<Index> idx(n), none;
  std::iota(idx.begin(), idx.end(), 0);
  std::vector<Index> poly{0, 1, 2, 3};
  pgpu::DomainDivider div(p.data(), nullptr, idx, none, poly);
  auto got = div.choose_coarse_points(10 * n).first;
  CHECK(static_cast<Index>(got.size()) == n);
  CHECK(std::equal(poly.begin(), poly.end(), got.begin()));
  CHECK(std::is_sorted(got.begin() + 4, got.end()));
  CHECK(static_cast<Index>(std::set<Index>(got.begin(), got.end()).size()) == n);
}

// The split sizes shared by the host and device dividers.
static void check_split_sizes() {
  for (Index n = 1025; n < 200000; n = n * 3 / 2 + 7) {
    Index lp, mid, rp;
    pgpu::overlap_split_sizes(n, lp, mid, rp);
    CHECK(0 < lp && lp <= mid && mid <= rp && rp < n);
    CHECK(rp + (n - lp) >= n);  // the halves cover the domain
  }
  for (Index n = 0; n < 100; ++n) {
    const Index m = pgpu::cluster_split(n);
    Index best = 0, bestd = n;
    for (Index i = 1; i < n; ++i) {
      const Index di = std::llabs(2 * i - n);
      if (di < bestd || (di == bestd && i % 2 == 0)) {
        best = i;
        bestd = di;
      }
    }
    CHECK(m == best);
  }
}

// The data-parallel split of large point sets gives the same domains and coarse points as the
// sequential selection.
static void check_parallel_splits(Index n_points, unsigned seed) {
  std::mt19937 gen(seed);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::vector<double> pts(3 * n_points);
  for (auto& v : pts) v = u(gen);
  std::vector<Index> idx(n_points), none;
  std::iota(idx.begin(), idx.end(), 0);
  std::vector<Index> poly{0, 1, 2, 3};
  pgpu::set_parallel_split_min(Index{1} << 40);
  pgpu::DomainDivider seq(pts.data(), nullptr, idx, none, poly);
  auto cseq = seq.choose_coarse_points(n_points / 10).first;
  pgpu::set_parallel_split_min(2000);
  pgpu::DomainDivider par(pts.data(), nullptr, idx, none, poly);
  auto cpar = par.choose_coarse_points(n_points / 10).first;
  pgpu::set_parallel_split_min(262144);
  CHECK(seq.domains().size() == par.domains().size());
  for (size_t k = 0; k < std::min(seq.domains().size(), par.domains().size()); ++k) {
    CHECK(seq.domains()[k].point_indices == par.domains()[k].point_indices);
    CHECK(seq.domains()[k].inner_point == par.domains()[k].inner_point);
  }
  std::sort(cseq.begin(), cseq.end());
  std::sort(cpar.begin(), cpar.end());
  CHECK(cseq == cpar);
}

static void check_lagrange() {
  std::mt19937 gen(11);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  for (int degree = 0; degree <= 2; ++degree) {
    const int l = (degree + 1) * (degree + 2) * (degree + 3) / 6;
    std::vector<double> pts(3 * 200);
    for (auto& v : pts) v = u(gen);
    const auto idx = pgpu::unisolvent_point_set(pts.data(), 200, degree);
    CHECK(static_cast<int>(idx.size()) == l);
    std::vector<double> pp;
    for (auto i : idx)
      for (int k = 0; k < 3; ++k) pp.push_back(pts[3 * i + k]);
    const auto coeffs = pgpu::lagrange_coeffs(degree, pp.data(), l);
    // L_c(p_r) = sum_k m_k(p_r) coeffs[k][c] = delta_rc.
    double err = 0;
    for (int r = 0; r < l; ++r) {
      double m[10];
      pgpu::monomial_row(degree, pp.data() + 3 * r, m);
      for (int c = 0; c < l; ++c) {
        double v = 0;
        for (int k = 0; k < l; ++k) v += m[k] * coeffs[k * l + c];
        err = std::max(err, std::fabs(v - (r == c ? 1.0 : 0.0)));
      }
    }
    CHECK(err < 1e-12);
  }
  {
    // Degree 1 at one point x and one gradient point y: rows m(x), dm/dx(y), dm/dy(y), dm/dz(y).
    const double x[3] = {0.3, -0.2, 0.7};
    std::vector<double> rows = {1, x[0], x[1], x[2], 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    const auto coeffs = pgpu::lagrange_coeffs_of(rows, 4);
    double err = 0;
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        double v = 0;
        for (int k = 0; k < 4; ++k) v += rows[r * 4 + k] * coeffs[k * 4 + c];
        err = std::max(err, std::fabs(v - (r == c ? 1.0 : 0.0)));
      }
    CHECK(err < 1e-12);
  }
  {
    const double same[12] = {0.1, 0.2, 0.3, 0.1, 0.2, 0.3, 0.5, 0.5, 0.5, 0.9, 0.1, 0.4};
    bool thrown = false;
    try {
      pgpu::lagrange_coeffs(1, same, 4);
    } catch (const pgpu::Error&) {
      thrown = true;
    }
    CHECK(thrown);
  }
}

int main() {
  check_lagrange();
  check_parallel_splits(30000, 7);
  check_divider(10000, 10000, 10, 1);
  check_divider(20000, 0, 4, 2);
  check_divider(5000, 3000, 1, 3);
  check_coarse_equivalence(5000, 700, 4);
  check_coarse_equivalence(20000, 2048, 5);
  check_coarse_equivalence(3000, 1500, 6);
  check_coarse_saturation(200, 8);
  check_split_sizes();
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
