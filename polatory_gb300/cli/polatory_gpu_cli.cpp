// polatory-gpu: the reference's command-line `fit` and `evaluate` (cli/fit_command.cpp:44-93,
// cli/evaluate_command.cpp:29-51) on the GPU library, through its C ABI only. Same options, the
// same table format (cli reads polatory::read_table: whitespace or comma separated, '#' comment
// lines; writes space-separated shortest round-trip numbers) and the reference's interpolant
// file format, so files move between the two programs. Three dimensions only.
//
//   polatory-gpu fit --in FILE --dim 3 (--model FILE | --rbf NAME PARAMS [aniso A11 .. A33] ...
//                    [--nug NUG] [--deg D]) --tol TOL [--grad-tol TOL] [--max-iter N] [--acc ACC]
//                    [--grad-acc ACC] [--ineq | --reduce] [--initial FILE] --out FILE
//   polatory-gpu evaluate --in FILE --points FILE --dim 3 [--grads] [--acc ACC] [--grad-acc ACC]
//                         --out FILE
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "polatory_gpu.h"

namespace {

const double kInf = std::numeric_limits<double>::infinity();

void check(int rc) {
  if (rc != PGPU_OK) throw std::runtime_error(pgpu_last_error());
}

struct Table {
  std::vector<double> v;
  size_t cols = 0;
  size_t rows() const { return cols ? v.size() / cols : 0; }
  double at(size_t r, size_t c) const { return v[r * cols + c]; }
};

double to_double(const std::string& s) {
  double x = std::numeric_limits<double>::quiet_NaN();
  const char* b = s.data();
  if (!s.empty() && *b == '+') ++b;
  std::from_chars(b, s.data() + s.size(), x);
  return x;
}

std::string trim(const std::string& s) {
  size_t b = 0, e = s.size();
  while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
  while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
  return s.substr(b, e - b);
}

// polatory::read_table (table.hpp:16-59): cells split at any of " \t,", lines starting with '#'
// skipped, rows with another column count skipped with a warning.
Table read_table(const std::string& filename) {
  std::ifstream ifs(filename);
  if (!ifs) throw std::runtime_error("cannot open file '" + filename + "'");
  Table t;
  std::string line;
  int line_no = 0;
  while (std::getline(ifs, line)) {
    ++line_no;
    if (line.rfind("#", 0) == 0) continue;
    std::vector<std::string> row;
    std::string cell;
    for (char ch : line) {
      if (ch == ' ' || ch == '\t' || ch == ',') {
        row.push_back(cell);
        cell.clear();
      } else {
        cell.push_back(ch);
      }
    }
    row.push_back(cell);
    if (t.cols == 0) {
      t.cols = row.size();
    } else if (row.size() != t.cols) {
      std::cerr << "warning: skipping line " << line_no << " with a different number of columns\n";
      continue;
    }
    for (const auto& c : row) t.v.push_back(to_double(trim(c)));
  }
  if (t.cols == 0) throw std::runtime_error("file '" + filename + "' is empty");
  return t;
}

// polatory::write_table (table.hpp:62-79): space-separated, shortest round-trip representation.
void write_table(const std::string& filename, const std::vector<double>& v, size_t cols) {
  std::ofstream ofs(filename);
  if (!ofs) throw std::runtime_error("cannot open file '" + filename + "'");
  char buf[32];
  for (size_t r = 0; r < v.size() / cols; ++r) {
    for (size_t c = 0; c < cols; ++c) {
      auto res = std::to_chars(buf, buf + sizeof(buf), v[r * cols + c]);
      ofs.write(buf, res.ptr - buf);
      if (c + 1 != cols) ofs << ' ';
    }
    ofs << '\n';
  }
}

// Reference short names (rbf/make_rbf.hpp:28-43).
const std::map<std::string, int> kKinds{
    {"bh2", PGPU_RBF_BH2}, {"bh3", PGPU_RBF_BH3}, {"cub", PGPU_RBF_CUB}, {"exp", PGPU_RBF_EXP},
    {"gau", PGPU_RBF_GAU}, {"gc3", PGPU_RBF_GC3}, {"gc5", PGPU_RBF_GC5}, {"gc7", PGPU_RBF_GC7},
    {"gc9", PGPU_RBF_GC9}, {"sph", PGPU_RBF_SPH}, {"sp3", PGPU_RBF_SP3}, {"sp5", PGPU_RBF_SP5},
    {"sp7", PGPU_RBF_SP7}, {"sp9", PGPU_RBF_SP9}, {"th2", PGPU_RBF_TH2}, {"th3", PGPU_RBF_TH3}};

bool is_identifier(const std::string& t) {
  static const std::regex re{"[A-Z_a-z][0-9A-Z_a-z]*"};
  return std::regex_match(t, re);
}
bool is_number(const std::string& t) {
  static const std::regex re{"-?([0-9]+\\.?|[0-9]*\\.[0-9]+)([Ee][+-]?[0-9]+)?"};
  return std::regex_match(t, re);
}

// examples/common/make_model.hpp:32-83: NAME PARAMS [aniso A11 .. A33] ..., row-major anisotropy.
pgpu_model make_model(const std::vector<std::string>& args, double nugget, int degree) {
  pgpu_model m{};
  size_t i = 0;
  while (i < args.size() && is_identifier(args[i])) {
    auto k = kKinds.find(args[i]);
    if (k == kKinds.end()) throw std::runtime_error("unknown RBF name: '" + args[i] + "'");
    if (m.n_rbfs == PGPU_MAX_RBFS) throw std::runtime_error("too many RBFs");
    ++i;
    pgpu_rbf& r = m.rbfs[m.n_rbfs++];
    r.kind = k->second;
    std::vector<double> p;
    while (i < args.size() && is_number(args[i])) p.push_back(to_double(args[i++]));
    const bool polyharmonic = r.kind == PGPU_RBF_BH2 || r.kind == PGPU_RBF_BH3 ||
                              r.kind == PGPU_RBF_TH2 || r.kind == PGPU_RBF_TH3;
    // Defaults of the polyharmonic splines: scale 1, c 0 (rbf/polyharmonic_*.hpp).
    r.params[0] = p.size() > 0 ? p[0] : (polyharmonic ? 1.0 : NAN);
    r.params[1] = p.size() > 1 ? p[1] : (polyharmonic ? 0.0 : NAN);
    // Polyharmonic splines take [SCALE [C]], covariance functions PSILL RANGE.
    if (p.size() > 2 || (!polyharmonic && p.size() != 2))
      throw std::invalid_argument("wrong number of parameters for '" + k->first + "'");
    for (int a = 0; a < 9; ++a) r.aniso[a] = (a % 4 == 0) ? 1.0 : 0.0;
    while (i < args.size() && args[i] == "aniso") {
      ++i;
      for (int a = 0; a < 9; ++a) {
        if (i >= args.size() || !is_number(args[i]))
          throw std::runtime_error(i >= args.size() ? "unexpected end of input"
                                                    : "unexpected token: '" + args[i] + "'");
        r.aniso[a] = to_double(args[i++]);
      }
    }
  }
  if (i != args.size()) throw std::runtime_error("unexpected token: '" + args[i] + "'");
  if (m.n_rbfs == 0) throw std::runtime_error("unexpected end of input");
  // Model<Dim>::kMinRequiredPolyDegree (-2): the lowest degree the RBFs allow.
  if (degree == -2) {
    int cpd = 0;
    for (int r = 0; r < m.n_rbfs; ++r) {
      int c = 0;
      check(pgpu_rbf_cpd_order(&m.rbfs[r], &c));
      cpd = std::max(cpd, c);
    }
    degree = cpd - 1;
  }
  m.poly_degree = degree;
  m.nugget = nugget;
  check(pgpu_model_validate(&m));
  return m;
}

struct Args {
  std::map<std::string, std::vector<std::string>> opts;
  bool has(const std::string& k) const { return opts.count(k) != 0; }
  std::string str(const std::string& k) const {
    auto it = opts.find(k);
    if (it == opts.end() || it->second.empty()) throw std::invalid_argument("missing --" + k);
    return it->second[0];
  }
  double num(const std::string& k, double def) const { return has(k) ? to_double(str(k)) : def; }
};

Args parse(int argc, char** argv, int first, const std::vector<std::string>& flags) {
  Args a;
  std::string key;
  for (int i = first; i < argc; ++i) {
    std::string t = argv[i];
    if (t.rfind("--", 0) == 0) {
      key = t.substr(2);
      a.opts[key];
      for (const auto& f : flags)
        if (f == key) key.clear();
    } else if (!key.empty()) {
      a.opts[key].push_back(t);
    } else {
      throw std::invalid_argument("unexpected argument: '" + t + "'");
    }
  }
  return a;
}

void require_dim3(const Args& a) {
  if (a.str("dim") != "3") throw std::invalid_argument("only --dim 3 is supported");
}

int run_fit(const Args& a) {
  require_dim3(a);
  if (a.has("grad-in") && a.has("ineq"))
    throw std::runtime_error("--grad-in cannot be used in conjunction with --ineq");
  if (a.has("initial") && a.has("reduce"))
    throw std::runtime_error("--initial cannot be used in conjunction with --reduce");
  if (a.has("grad-in")) throw std::runtime_error("gradient data points are not supported yet");
  const Table t = read_table(a.str("in"));
  const bool ineq = a.has("ineq");
  if (t.cols < (ineq ? 6u : 4u)) throw std::runtime_error("too few columns in '" + a.str("in") + "'");
  const size_t n = t.rows();
  std::vector<double> pts(3 * n), vals(n), lb(n), ub(n);
  for (size_t r = 0; r < n; ++r) {
    for (int k = 0; k < 3; ++k) pts[3 * r + k] = t.at(r, k);
    vals[r] = t.at(r, 3);
    if (ineq) {
      lb[r] = t.at(r, 4);
      ub[r] = t.at(r, 5);
    }
  }
  pgpu_interpolant* it = nullptr;
  // The library reads and writes models inside interpolant files only.
  if (a.has("model")) throw std::runtime_error("--model files are not supported; give --rbf");
  if (!a.has("rbf")) throw std::invalid_argument("missing --rbf");
  pgpu_model m = make_model(a.opts.at("rbf"), a.num("nug", 0.0),
                            a.has("deg") ? static_cast<int>(a.num("deg", 0)) : -2);
  check(pgpu_interpolant_create(&m, &it));
  const double tol = a.num("tol", NAN);
  const double grad_tol = a.num("grad-tol", -1.0) == -1.0 ? tol : a.num("grad-tol", tol);
  const int max_iter = static_cast<int>(a.num("max-iter", 100));
  const double acc = a.num("acc", kInf), grad_acc = a.num("grad-acc", kInf);
  pgpu_interpolant* initial = nullptr;
  if (a.has("initial")) check(pgpu_interpolant_load(a.str("initial").c_str(), &initial));
  int rc;
  if (ineq)
    rc = pgpu_interpolant_fit_inequality(it, pts.data(), n, vals.data(), lb.data(), ub.data(), tol,
                                         max_iter, acc);
  else if (a.has("reduce"))
    rc = pgpu_interpolant_fit_incrementally(it, pts.data(), n, nullptr, 0, vals.data(), tol,
                                            grad_tol, max_iter, acc, grad_acc);
  else
    rc = pgpu_interpolant_fit(it, pts.data(), n, nullptr, 0, vals.data(), tol, grad_tol, max_iter,
                              acc, grad_acc, initial);
  if (initial) pgpu_interpolant_destroy(initial);
  if (rc != PGPU_OK) {
    const std::string msg = pgpu_last_error();
    pgpu_interpolant_destroy(it);
    throw std::runtime_error(msg);
  }
  check(pgpu_interpolant_save(it, a.str("out").c_str()));
  pgpu_interpolant_destroy(it);
  return 0;
}

int run_evaluate(const Args& a) {
  require_dim3(a);
  pgpu_interpolant* it = nullptr;
  check(pgpu_interpolant_load(a.str("in").c_str(), &it));
  const Table t = read_table(a.str("points"));
  if (t.cols < 3) throw std::runtime_error("too few columns in '" + a.str("points") + "'");
  const size_t n = t.rows();
  std::vector<double> pts(3 * n);
  for (size_t r = 0; r < n; ++r)
    for (int k = 0; k < 3; ++k) pts[3 * r + k] = t.at(r, k);
  const bool grads = a.has("grads");
  std::vector<double> out(n + (grads ? 3 * n : 0));
  const double acc = a.num("acc", kInf), grad_acc = a.num("grad-acc", kInf);
  const int rc = pgpu_interpolant_evaluate(it, pts.data(), n, grads ? pts.data() : nullptr,
                                           grads ? n : 0, acc, grad_acc, out.data());
  if (rc != PGPU_OK) {
    const std::string msg = pgpu_last_error();
    pgpu_interpolant_destroy(it);
    throw std::runtime_error(msg);
  }
  pgpu_interpolant_destroy(it);
  const size_t cols = grads ? 7 : 4;
  std::vector<double> table(n * cols);
  for (size_t r = 0; r < n; ++r) {
    for (int k = 0; k < 3; ++k) table[r * cols + k] = pts[3 * r + k];
    table[r * cols + 3] = out[r];
    if (grads)
      for (int k = 0; k < 3; ++k) table[r * cols + 4 + k] = out[n + 3 * r + k];
  }
  write_table(a.str("out"), table, cols);
  return 0;
}

void usage() {
  std::cout << "usage: polatory-gpu fit --in FILE --dim 3 --rbf NAME PARAMS [aniso A11 .. A33] "
               "[--nug NUG] [--deg D] --tol TOL [--grad-tol TOL] [--max-iter N] [--acc ACC] "
               "[--grad-acc ACC] [--ineq | --reduce] [--initial FILE] --out FILE\n"
               "       polatory-gpu evaluate --in FILE --points FILE --dim 3 [--grads] [--acc ACC] "
               "[--grad-acc ACC] --out FILE\n";
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2 || std::strcmp(argv[1], "--help") == 0 || std::strcmp(argv[1], "help") == 0) {
    usage();
    return argc < 2 ? 1 : 0;
  }
  try {
    const std::string cmd = argv[1];
    if (cmd == "fit") return run_fit(parse(argc, argv, 2, {"ineq", "reduce"}));
    if (cmd == "evaluate") return run_evaluate(parse(argc, argv, 2, {"grads"}));
    usage();
    return 1;
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << '\n';
    return 1;
  }
}
