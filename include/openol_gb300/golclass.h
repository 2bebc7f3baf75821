/*
 * golclass.h (drop-in) -- the device containers of the reference's
 * include/golclass.h (cuda::unique_ptr with a cudaFree deleter,
 * cuda::make_unique, ol::gObject, Object2cuda, cpu2cuda / cuda2cpu;
 * golclass.h:9-121), restated so that caller code written against the
 * reference compiles unchanged on top of libolgb300.so.
 */
#ifndef OLGB300_GOLCLASS_H
#define OLGB300_GOLCLASS_H
#include <cuda_runtime_api.h>

#include <memory>
#include <sstream>
#include <stdexcept>
#include <type_traits>

#include "olclass.h"

#define CHECK_CUDA_ERROR(e) (cuda::check_error(e, __FILE__, __LINE__))
namespace cuda {
template <typename F, typename N>
void check_error(const ::cudaError_t e, F &&f, N &&n)
{
    if (e != ::cudaSuccess) {
        std::ostringstream s;
        s << "CUDA call failed at " << f << ":" << n << " -- " << ::cudaGetErrorString(e) << " ["
          << ::cudaGetErrorName(e) << ", code " << static_cast<int>(e) << "]";
        throw std::runtime_error{s.str()};
    }
}
struct deleter {
    void operator()(void *p) const { CHECK_CUDA_ERROR(::cudaFree(p)); }
};
template <typename T>
using unique_ptr = std::unique_ptr<T, deleter>;

template <typename T>
typename std::enable_if<std::is_array<T>::value, cuda::unique_ptr<T>>::type make_unique(const std::size_t n)
{
    using U = typename std::remove_extent<T>::type;
    U *p;
    CHECK_CUDA_ERROR(::cudaMalloc(reinterpret_cast<void **>(&p), sizeof(U) * n));
    return cuda::unique_ptr<T>{p};
}
} // namespace cuda

namespace ol {
template <typename _Tp>
struct gObject {
    int size = 0;
    cuda::unique_ptr<ol::Vect3<_Tp>[]> points;
    gObject() {}
    explicit gObject(int N) : size(N), points(cuda::make_unique<ol::Vect3<_Tp>[]>(N)) {}
};

template <typename _Tp>
gObject<_Tp> Object2cuda(ol::Object<_Tp> &obj)
{
    gObject<_Tp> g(obj.size);
    CHECK_CUDA_ERROR(cudaMemcpy(g.points.get(), obj.points.get(), sizeof(obj.points[0]) * obj.size, cudaMemcpyHostToDevice));
    return g;
}

template <typename _Tsrc, typename _Tdst>
void cpu2cuda(std::unique_ptr<_Tsrc[]> &src, cuda::unique_ptr<_Tdst[]> &dst, int size)
{
    if (!dst) dst = cuda::make_unique<_Tdst[]>(size);
    CHECK_CUDA_ERROR(cudaMemcpy(dst.get(), src.get(), size * sizeof(_Tsrc), cudaMemcpyHostToDevice));
}

template <typename _Tsrc, typename _Tdst>
void cuda2cpu(cuda::unique_ptr<_Tsrc[]> &src, std::unique_ptr<_Tdst[]> &dst, int size)
{
    if (!dst) dst = std::make_unique<_Tdst[]>(size);
    CHECK_CUDA_ERROR(cudaMemcpy(dst.get(), src.get(), size * sizeof(_Tsrc), cudaMemcpyDeviceToHost));
}
} // namespace ol
#endif
