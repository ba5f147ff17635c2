// Host-side set-up of the RAS preconditioner: unisolvent polynomial points, Lagrange basis
// coefficients and the overlapping domain decomposition with coarse-point selection.
#pragma once

#include <utility>
#include <vector>

#include "common.hpp"

namespace pgpu {

// One overlapping domain: indices into the full point arrays, value points first (the
// polynomial points lead the list) and inner flags (points whose solution the domain owns).
struct Domain {
  std::vector<Index> point_indices;
  std::vector<Index> grad_point_indices;
  std::vector<char> inner_point;
  std::vector<char> inner_grad_point;
  Index num_points() const { return static_cast<Index>(point_indices.size()); }
  Index num_grad_points() const { return static_cast<Index>(grad_point_indices.size()); }
};

// Restatement of preconditioner::DomainDivider (include/polatory/preconditioner/
// domain_divider.hpp:18-321): recursive splits along the widest axes with an overlap quota of
// 0.5 down to at most 1024 points (gradient points count three times); coarse points chosen by
// priority-queue bisection. points/grad_points: host xyz rows of the full point sets.
// Point sets of at least n points are split data-parallel (same results as the sequential
// selection); the tests lower it to cover that path on small inputs.
void set_parallel_split_min(Index n);

// Sizes of the two overlapping halves of a domain of n value points (domain_divider.hpp:
// 199-213): in the domain's sorted order the left half takes positions [0, right_part), the
// right half [left_part, n); positions below mid stay inner on the left, the rest on the right.
void overlap_split_sizes(Index n, Index& left_part, Index& mid, Index& right_part);

// Split position of a coarse-point cluster of n value points (domain_divider.hpp:82-88).
Index cluster_split(Index n);

class DomainDivider {
 public:
  DomainDivider(const double* points, const double* grad_points,
                const std::vector<Index>& point_indices,
                const std::vector<Index>& grad_point_indices,
                const std::vector<Index>& poly_point_indices);

  // Coarse points: the polynomial points, then the cluster centres in ascending index order.
  std::pair<std::vector<Index>, std::vector<Index>> choose_coarse_points(Index n_coarse) const;

  // The coarse-point selection alone: it reads only the point sets, so it can run while the
  // division of the same sets runs elsewhere.
  static std::pair<std::vector<Index>, std::vector<Index>> choose_coarse_points(
      const double* points, const double* grad_points, const std::vector<Index>& point_indices,
      const std::vector<Index>& grad_point_indices,
      const std::vector<Index>& poly_point_indices, Index n_coarse);

  std::vector<Domain>& domains() { return domains_; }

  static constexpr double kOverlapQuota = 0.5;
  static constexpr Index kMaxLeafSize = 1024;

 private:
  const double* points_;
  const double* grad_points_;
  std::vector<Index> point_idcs_;
  std::vector<Index> grad_point_idcs_;
  std::vector<Index> poly_point_idcs_;
  std::vector<Domain> domains_;
};

// Monomial basis rows of one point (3-D, degree <= 2; monomial_basis.hpp:171-247 order).
void monomial_row(int degree, const double* p, double* out);

// polynomial::UnisolventPointSet (unisolvent_point_set.hpp:25-66): 100 random trials of l
// distinct points (std::mt19937 default seed, uniform_int_distribution), keeping the set with
// the best reciprocal condition number. Returns sorted indices. Throws runtime error
// "could not find a unisolvent set of points" when no trial is invertible.
std::vector<Index> unisolvent_point_set(const double* points, Index n, int degree);

// Inverse of the monomial matrix of l unisolvent points (lagrange_basis.hpp:28-45).
// Throws invalid_argument "the set of points is not unisolvent".
std::vector<double> lagrange_coeffs(int degree, const double* poly_points, Index l,
                                    double* rcond_out = nullptr);
// The same from the l x l matrix of monomial rows (value rows or gradient-component rows; the
// special case of lagrange_basis.hpp:36-37: one point and one gradient point at degree 1).
std::vector<double> lagrange_coeffs_of(const std::vector<double>& rows, Index l);

}  // namespace pgpu
