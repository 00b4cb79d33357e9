// Core types, constants and small vector math for the GB300 stepping loop.
//
// Everything here is usable from host and device code. Floating-point
// expressions are spelled out in the same operation order as the reference
// (explicit fma where it uses std::fma, plain multiply/add elsewhere) so that
// the FP64 build reproduces the reference's host results bit for bit when the
// device code is compiled without FMA contraction (-fmad=false).
#pragma once

#include <cmath>
#include <cstdint>

#include "Libm.hh"
#include "Macros.hh"

#ifndef GBX_PHYS_REAL
#    define GBX_PHYS_REAL double
#endif

namespace gbx
{
//! Precision of the physics arithmetic (energies, cross sections, ...)
using real_type = GBX_PHYS_REAL;
//! Precision of positions, directions and geometric distances (always FP64)
using geo_real = double;
using size_type = std::uint32_t;

//! "Invalid" marker for all 32-bit IDs
constexpr size_type invalid_id = static_cast<size_type>(-1);

namespace constants
{
// Mathematical constants (corecel/Constants.hh)
constexpr double pi = 3.14159265358979323846;
// CGS units: cm, g, s; energies in MeV where labelled (celeritas/Units.hh)
constexpr double centimeter = 1;
constexpr double meter = 100 * centimeter;
constexpr double millimeter = 0.1 * centimeter;
constexpr double second = 1;
constexpr double gram = 1;
constexpr double gauss = 1;
constexpr double tesla = 10000 * gauss;
constexpr double barn = 1e-24 * centimeter * centimeter;
// CODATA 2018 physical constants (celeritas/Constants.hh)
constexpr double c_light = 299792458. * meter / second;
constexpr double alpha_fine_structure = 7.2973525693e-3;
constexpr double atomic_mass = 1.66053906660e-24 * gram;
constexpr double r_electron = 2.8179403262e-15 * meter;
constexpr double lambdabar_electron = 3.8615926796e-13 * meter;
constexpr double na_avogadro = 6.02214076e23;
}  // namespace constants

//---------------------------------------------------------------------------//
// Integer power by recursive squaring: ipow<N>(v) multiplies in the order
// v * ipow<(N-1)/2> * ipow<(N-1)/2> for odd N, ipow<N/2> * ipow<N/2> for even.
template<unsigned int N, class T>
GBX_FORCEINLINE constexpr T ipow(T v)
{
    if constexpr (N == 0)
    {
        return T(1);
    }
    else if constexpr (N % 2 == 0)
    {
        return ipow<N / 2>(v) * ipow<N / 2>(v);
    }
    else
    {
        return v * ipow<(N - 1) / 2>(v) * ipow<(N - 1) / 2>(v);
    }
}

template<class T>
GBX_FORCEINLINE constexpr T min_of(T a, T b)
{
    return b < a ? b : a;
}
template<class T>
GBX_FORCEINLINE constexpr T max_of(T a, T b)
{
    return a < b ? b : a;
}

GBX_FORCEINLINE double gbx_fma(double a, double b, double c)
{
    return ::fma(a, b, c);
}
GBX_FORCEINLINE float gbx_fma(float a, float b, float c)
{
    return ::fmaf(a, b, c);
}

//---------------------------------------------------------------------------//
// Three-vector
//---------------------------------------------------------------------------//
template<class T>
struct Vec3
{
    T x, y, z;

    GBX_FORCEINLINE T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    GBX_FORCEINLINE T operator[](int i) const
    {
        return i == 0 ? x : (i == 1 ? y : z);
    }
};
using Real3 = Vec3<double>;

//! Dot product accumulated with fma in index order
template<class T>
GBX_FORCEINLINE T dot_product(Vec3<T> const& a, Vec3<T> const& b)
{
    T result{0};
    result = gbx_fma(a.x, b.x, result);
    result = gbx_fma(a.y, b.y, result);
    result = gbx_fma(a.z, b.z, result);
    return result;
}

template<class T>
GBX_FORCEINLINE T norm(Vec3<T> const& v)
{
    return std::sqrt(dot_product(v, v));
}

template<class T>
GBX_FORCEINLINE Vec3<T> make_unit_vector(Vec3<T> const& v)
{
    T const scale = T(1) / norm(v);
    return {v.x * scale, v.y * scale, v.z * scale};
}

//! Geometry direction from a physics direction. The geometry solves its
//! surface intersections for a unit direction (the cylinder quadratic takes
//! dx^2 + dy^2 as 1 - dz^2); a direction computed in FP32 is a unit vector
//! only to FP32 rounding (|d|^2 - 1 up to ~1e-7), which moves the roots by
//! ~1e-7 of the distance, far more than the bump that decides which volume
//! lies across a crossing. FP32 directions are therefore renormalized in
//! FP64; FP64 directions pass through unchanged.
template<class T>
GBX_FORCEINLINE Vec3<double> to_geo_dir(Vec3<T> const& d)
{
    Vec3<double> r{double(d.x), double(d.y), double(d.z)};
    if constexpr (sizeof(T) < sizeof(double))
    {
        r = make_unit_vector(r);
    }
    return r;
}

//! y <- a * x + y, with fma per component
template<class T>
GBX_FORCEINLINE void axpy(T a, Vec3<T> const& x, Vec3<T>* y)
{
    y->x = gbx_fma(a, x.x, y->x);
    y->y = gbx_fma(a, x.y, y->y);
    y->z = gbx_fma(a, x.z, y->z);
}

//! Unit vector from polar cosine and azimuthal angle
template<class T>
GBX_FORCEINLINE Vec3<T> from_spherical(T costheta, T phi)
{
    T const sintheta = std::sqrt(1 - costheta * costheta);
    return {sintheta * libm::cos(phi), sintheta * libm::sin(phi), costheta};
}

//! Rotate a direction given in the frame whose z axis is 'rot' into the lab
//! frame (same branch structure as the reference's rotate()).
template<class T>
GBX_FORCEINLINE Vec3<T> rotate(Vec3<T> const& dir, Vec3<T> const& rot)
{
    constexpr T min_accurate_sintheta = sizeof(T) == 8 ? T(0.005) : T(0.07);
    T sintheta = std::sqrt(1 - ipow<2>(rot.z));
    T cosphi;
    T sinphi;
    if (sintheta >= min_accurate_sintheta)
    {
        T const inv_sintheta = 1 / (sintheta);
        cosphi = rot.x * inv_sintheta;
        sinphi = rot.y * inv_sintheta;
    }
    else if (sintheta > 0)
    {
        cosphi = rot.x / std::sqrt(ipow<2>(rot.x) + ipow<2>(rot.y));
        sinphi = std::sqrt(1 - ipow<2>(cosphi));
    }
    else
    {
        cosphi = 1;
        sinphi = 0;
    }
    Vec3<T> result{(rot.z * dir.x + sintheta * dir.z) * cosphi - sinphi * dir.y,
                   (rot.z * dir.x + sintheta * dir.z) * sinphi + cosphi * dir.y,
                   -sintheta * dir.x + rot.z * dir.z};
    return make_unit_vector(result);
}

//! Direction of a*p_a - b*p_b, normalized (momentum conservation)
template<class T>
GBX_FORCEINLINE Vec3<T> calc_exiting_direction(T inc_mag,
                                               Vec3<T> const& inc_dir,
                                               T out_mag,
                                               Vec3<T> const& out_dir)
{
    Vec3<T> r{inc_dir.x * inc_mag - out_dir.x * out_mag,
              inc_dir.y * inc_mag - out_dir.y * out_mag,
              inc_dir.z * inc_mag - out_dir.z * out_mag};
    return make_unit_vector(r);
}

//! Horner evaluation of c[0] + x (c[1] + x (c[2] + ...)) with fma
template<int N, class T>
GBX_FORCEINLINE T poly_eval(T const* c, T x)
{
    T result = c[N];
    for (int i = N - 1; i >= 0; --i)
    {
        result = gbx_fma(x, result, c[i]);
    }
    return result;
}

}  // namespace gbx
