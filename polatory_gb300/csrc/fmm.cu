// Interpolation-based FMM (placeholder until the tree and passes land): reports no support, so
// every evaluator uses the exact direct backend.
#include "fmm.hpp"

namespace pgpu {

template <class T>
struct Fmm<T>::Impl {};

template <class T>
bool Fmm<T>::supported(int) { return false; }

template <class T>
Fmm<T>::Fmm(int, const KParams<T>&, const Mat3&, const double*, double, double) : impl_(new Impl) {}

template <class T>
Fmm<T>::~Fmm() { delete impl_; }

template <class T>
void Fmm<T>::set_config(const FarFieldConfig&) {}
template <class T>
void Fmm<T>::set_points(const P4<T>*, Index, const P4<T>*, Index) {}
template <class T>
void Fmm<T>::set_sources(const P4<T>*, Index, const P4<T>*, Index) {}
template <class T>
void Fmm<T>::set_targets(const P4<T>*, Index, const P4<T>*, Index) {}
template <class T>
void Fmm<T>::evaluate(const T*, const T*, double*, double*) {
  throw_runtime("FMM backend unavailable");
}
template <class T>
Index Fmm<T>::near_pairs() const { return 0; }

template class Fmm<double>;
template class Fmm<float>;

}  // namespace pgpu
