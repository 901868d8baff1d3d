// Stand-in for boost::math::quaternion<T> as so3g's src/Projection.cxx
// uses it -- TEST INFRASTRUCTURE for oracle/ref_engine.cpp.  Four
// contiguous components (the engine reinterprets double[4] as a
// quaternion), the component accessors and the Hamilton product, each
// component's four terms summed left to right.  Boost (1.87 in the
// reference's build) is not installed here, so the order of boost's own
// sums -- which decides the product's last bit -- is not pinned; the
// oracle uses the same left-to-right order.
#pragma once

namespace boost {
namespace math {

template <class T>
class quaternion {
public:
    quaternion(T a = T(), T b = T(), T c = T(), T d = T()) : a_(a), b_(b), c_(c), d_(d) {}
    T R_component_1() const { return a_; }
    T R_component_2() const { return b_; }
    T R_component_3() const { return c_; }
    T R_component_4() const { return d_; }
    quaternion operator*(const quaternion &q) const {
        return quaternion(a_ * q.a_ - b_ * q.b_ - c_ * q.c_ - d_ * q.d_,
                          a_ * q.b_ + b_ * q.a_ + c_ * q.d_ - d_ * q.c_,
                          a_ * q.c_ - b_ * q.d_ + c_ * q.a_ + d_ * q.b_,
                          a_ * q.d_ + b_ * q.c_ - c_ * q.b_ + d_ * q.a_);
    }

private:
    T a_, b_, c_, d_;
};

}  // namespace math
}  // namespace boost
