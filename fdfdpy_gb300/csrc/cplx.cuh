// Minimal complex arithmetic for the factor kernels (float and double).
#pragma once

#include <cuda_runtime.h>

namespace fdfd {

template <typename R>
struct alignas(2 * sizeof(R)) cplx {
    R x, y;
};
using c64 = cplx<float>;
using c128 = cplx<double>;

template <typename R>
__device__ __forceinline__ cplx<R> cmake(R x, R y) {
    cplx<R> c;
    c.x = x;
    c.y = y;
    return c;
}
template <typename R>
__device__ __forceinline__ cplx<R> cadd(cplx<R> a, cplx<R> b) {
    return cmake<R>(a.x + b.x, a.y + b.y);
}
template <typename R>
__device__ __forceinline__ cplx<R> csub(cplx<R> a, cplx<R> b) {
    return cmake<R>(a.x - b.x, a.y - b.y);
}
template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
    return cmake<R>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// acc += a * b
template <typename R>
__device__ __forceinline__ void cmac(cplx<R> &acc, cplx<R> a, cplx<R> b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
// acc -= a * b
template <typename R>
__device__ __forceinline__ void cmsub(cplx<R> &acc, cplx<R> a, cplx<R> b) {
    acc.x = fma(-a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(-a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}
template <typename R>
__device__ __forceinline__ R cabs2(cplx<R> a) {
    return fma(a.x, a.x, a.y * a.y);
}
// 1/b with the larger component factored out (no overflow for |b|^2).
template <typename R>
__device__ __forceinline__ cplx<R> crecip(cplx<R> b) {
    const R s = fmax(fabs(b.x), fabs(b.y));
    const R br = b.x / s, bi = b.y / s;
    const R d = s * fma(br, br, bi * bi);
    return cmake<R>(br / d, -bi / d);
}
template <typename T>
__device__ __forceinline__ T from_c128(double2 v, double s);
template <>
__device__ __forceinline__ c128 from_c128<c128>(double2 v, double s) {
    return cmake<double>(v.x * s, v.y * s);
}
template <>
__device__ __forceinline__ c64 from_c128<c64>(double2 v, double s) {
    return cmake<float>((float)(v.x * s), (float)(v.y * s));
}
template <typename R>
__device__ __forceinline__ double2 to_c128(cplx<R> v, double s) {
    return make_double2((double)v.x * s, (double)v.y * s);
}
template <typename T>
__device__ __forceinline__ T czero() {
    T z;
    z.x = 0;
    z.y = 0;
    return z;
}
template <typename T>
__device__ __forceinline__ T cone() {
    T z;
    z.x = 1;
    z.y = 0;
    return z;
}

}  // namespace fdfd
