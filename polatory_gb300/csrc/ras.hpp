// Multilevel restricted additive Schwarz (RAS) preconditioner on the device: the GPU form of
// preconditioner::RasPreconditioner (include/polatory/preconditioner/ras_preconditioner.hpp:
// 35-364) with FineGrid (fine_grid.hpp:36-195) and CoarseGrid (coarse_grid.hpp:19-159). The
// per-domain factors of Q^T A Q stay resident in HBM (the reference packs them into a temp
// file); all domains of a level are assembled, factorised and solved by batched kernels.
#pragma once

#include <map>
#include <memory>
#include <vector>

#include "common.hpp"
#include "evaluator.hpp"
#include "model.hpp"
#include "ras_host.hpp"

namespace pgpu {

// All domains of one level (or the single coarse domain) with their factors.
template <class T>
struct DomainBatch {
  Index n_dom = 0;
  int max_n = 0;                 // largest Q^T A Q size
  DevBuf<int> n;                 // Q^T A Q size per domain (m - l)
  DevBuf<int> ld;                // padded leading dimension (multiple of 32)
  DevBuf<Index> mat_off;         // offset of each factor in mats
  DevBuf<T> mats;                // column-major padded factors
  DevBuf<Index> pt_off;          // CSR offsets into pts
  DevBuf<Index> pts;             // global point indices, polynomial points first
  DevBuf<char> inner;            // inner flag per entry of pts
  DevBuf<int> info;              // per-domain count of modified pivots
  Index total_points = 0;
  double factor_flops = 0;       // sum of n^3 / 3
  double solve_bytes = 0;        // factor bytes read per solve (forward + backward sweeps)
};

template <class T>
class RasPreconditioner {
 public:
  // points_host / points_dev: the mu data points (xyz rows). Value points only.
  RasPreconditioner(const ModelDesc& model, const double* points_host, const double* points_dev,
                    Index mu, const Bbox3& bbox);
  // With sigma gradient points (grad_host / grad_dev): the system has mu + 3 sigma rows, the
  // gradient point j owning rows mu + 3 j .. + 2 (ras_preconditioner.hpp:56-189 with
  // grad_points). The levels are divided on the host (the device division is value-only).
  RasPreconditioner(const ModelDesc& model, const double* points_host, const double* points_dev,
                    Index mu, const double* grad_host, const double* grad_dev, Index sigma,
                    const Bbox3& bbox);
  // One domain holding all points, for the component tests of the fine and coarse grids:
  // `order` lists the points (the first l are the polynomial points), `inner` the fine-grid
  // inner flags per entry of `order`; coarse_inverse keeps the coarse grid as an explicit inverse.
  RasPreconditioner(const ModelDesc& model, const double* points_host, const double* points_dev,
                    Index mu, const std::vector<Index>& order, const std::vector<char>& inner,
                    bool coarse_inverse);
  ~RasPreconditioner();
  // Solves the test domain as the coarse grid (weights of every point and the polynomial
  // coefficients) or as a fine-grid domain (weights of the inner points).
  void solve_domain(bool coarse, const double* residuals, double* weights);

  // out (M) = RAS(v (M)), M = mu + 3 sigma + l (ras_preconditioner.hpp:191-250).
  void apply(const double* v, double* out);

  int levels() const { return n_levels_; }
  Index n_domains() const;
  Index size() const { return rows_ + l_; }

 private:
  void setup_polynomial(const double* points_host, const double* points_dev);
  void solve_level(int level, const double* residuals, double* weights);
  void update_residuals(int src_level, int trg_level, const double* weights, double* residuals);
  void orthogonalize(double* weights, double* residuals);
  template <class U>
  void build_batch(DomainBatch<U>& b, const std::vector<Domain>& domains);
  // The same from flattened device lists: sizes per domain, point indices and inner flags.
  template <class U>
  void build_batch(DomainBatch<U>& b, const std::vector<Index>& sizes, DevBuf<Index>&& pts,
                   DevBuf<char>&& inner);
  Evaluator<T>& evaluator(int src_level, int trg_level);

  // Fits with gradient points: the rows' positions and types and the gradient-point sets.
  void setup_rows(const double* points_host, const double* grad_host);
  template <class U>
  void build_batch_rows(DomainBatch<U>& b, const std::vector<Domain>& domains);

  ModelDesc model_;
  int l_;
  Index mu_;
  Index sigma_ = 0;
  Index rows_ = 0;  // mu + 3 sigma
  int n_levels_;
  Bbox3 bbox_;
  const double* points_dev_;
  const double* grad_dev_ = nullptr;
  std::vector<Index> poly_idcs_;
  std::vector<Index> poly_rows_;  // rows of the polynomial (Lagrange) functionals
  DevBuf<double> row_pos_;        // gradient fits: rows x 3
  DevBuf<int> row_type_;          // gradient fits: -1 value, 0-2 derivative axis
  std::vector<std::vector<Index>> grad_point_idcs_;
  std::vector<DevBuf<double>> level_grad_pts_dev_;
  std::vector<double> lagrange_coeffs_;  // l x l row-major inverse of the poly-point monomials
  std::vector<double> a11_;              // A restricted to the polynomial points (l x l)
  std::vector<std::vector<Index>> point_idcs_;
  std::vector<DevBuf<Index>> level_idx_dev_;
  std::vector<DevBuf<double>> level_pts_dev_;
  DevBuf<double> lagrange_;  // mu x l row-major
  DevBuf<double> u_;         // mu x l: sum_r K_r(p_k, x_i)
  DevBuf<double> v_;         // mu x l: A11 L_i
  std::vector<std::unique_ptr<DomainBatch<T>>> fine_;  // per level (index 0 unused)
  // The coarse grid is always factorised in FP64 and kept as an explicit inverse.
  DomainBatch<double> coarse_;
  DevBuf<double> coarse_inv_;  // n x n
  int coarse_n_ = 0;
  bool use_coarse_inverse_ = false;
  DevBuf<double> coarse_x_, coarse_g_, coarse_out_;
  DevBuf<double> p_;   // mu x l orthonormalised monomials (column-major)
  DevBuf<double> ap_;  // mu x l
  std::map<std::pair<int, int>, std::unique_ptr<Evaluator<T>>> evaluators_;
  DevBuf<double> work_res_, work_w_, work_tot_, work_src_w_, work_fit_;
};

// Component test of one RAS domain holding all n points (host buffers): `order` lists the
// points with the l polynomial points first, `inner` the fine-grid inner flags; solves rhs as the
// coarse grid (coarse, optionally through the explicit inverse) or as a fine-grid domain and
// writes the n + l weights. FP64 factors, or FP32 factors when mixed.
void ras_domain_solve(const ModelDesc& model, const double* points, Index n, const Index* order,
                      const unsigned char* inner, bool coarse, bool use_inverse, bool mixed,
                      const double* rhs, double* out);

}  // namespace pgpu
