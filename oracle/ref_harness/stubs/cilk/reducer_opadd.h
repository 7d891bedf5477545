#ifndef SG_REF_CILK_REDUCER_STUB_H_
#define SG_REF_CILK_REDUCER_STUB_H_
#include <atomic>
namespace cilk {
template <typename T>
class reducer_opadd {
 public:
  reducer_opadd() : v_(T()) {}
  explicit reducer_opadd(T v) : v_(v) {}
  reducer_opadd& operator+=(const T& x) {
#pragma omp critical(sg_reducer_opadd)
    v_ += x;
    return *this;
  }
  reducer_opadd& operator-=(const T& x) {
#pragma omp critical(sg_reducer_opadd)
    v_ -= x;
    return *this;
  }
  T get_value() const { return v_; }
  void set_value(T v) { v_ = v; }

 private:
  T v_;
};
}  // namespace cilk
#endif
