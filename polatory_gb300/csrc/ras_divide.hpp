// Device-side RAS set-up of one level: the overlapping domain division and the coarse-point
// selection of preconditioner::DomainDivider (include/polatory/preconditioner/
// domain_divider.hpp:18-321), for value points. Results equal the host restatement in
// ras_host.cpp (same domains in the same order, same inner flags, same coarse points in the
// same canonical order) whenever no two points of the level coincide; coincident points may
// trade places.
#pragma once

#include <vector>

#include "common.hpp"

namespace pgpu {

// The domains of one level, flattened in the host divider's order: per domain its size
// (polynomial points included), and the concatenated global point indices (polynomial points
// first, then ascending index) with their inner flags.
struct LevelDomains {
  std::vector<Index> sizes;
  DevBuf<Index> pts;
  DevBuf<char> inner;
};

class DeviceDivider {
 public:
  // coords: device xyz rows of all mu points as the division sees them (A-transformed for an
  // anisotropic model). poly: the polynomial points' global indices; every level list starts
  // with them.
  DeviceDivider(const double* coords, Index mu, const std::vector<Index>& poly);
  ~DeviceDivider();

  // Takes one level's point list (global indices, the polynomial points first, the rest
  // ascending) and ranks its coordinates per axis.
  void set_level(const std::vector<Index>& level);

  // Overlapping domains of at most 1024 points (domain_divider.hpp:161-276), in the order of the
  // reference's list (breadth first).
  void divide(LevelDomains& out);

  // Coarse points of the level (domain_divider.hpp:54-125): the polynomial points, then the
  // centres of the clusters in ascending index order.
  std::vector<Index> choose_coarse_points(Index n_coarse);

 private:
  struct Impl;
  Impl* impl_;
};

}  // namespace pgpu
