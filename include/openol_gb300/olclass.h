/*
 * olclass.h (drop-in) -- host point types of the reference's include/olclass.h
 * (Vect3 olclass.h:45-52, Object olclass.h:55-70), restated.
 */
#ifndef OLGB300_OLCLASS_H
#define OLGB300_OLCLASS_H
#include <memory>
namespace ol {
template <typename _Tp>
struct Vect3 {
    _Tp x, y, z;
    Vect3(_Tp x_, _Tp y_, _Tp z_) : x(x_), y(y_), z(z_) {}
    Vect3() {}
};
template <typename _Tp>
struct Object {
    int size = 0;
    std::unique_ptr<Vect3<_Tp>[]> points;
    Object() {}
    explicit Object(int N) : size(N), points(std::make_unique<Vect3<_Tp>[]>(N)) {}
    Vect3<_Tp> &operator[](int n) { return points[n]; }
};
} // namespace ol
#endif
