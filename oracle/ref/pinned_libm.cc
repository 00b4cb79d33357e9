// Pins the C library's elementary functions of the reference build to
// correctly rounded ones.
//
// The reference calls exp, log, sin, cos (or sincos, which the compiler forms
// from a sin and a cos of the same argument), tanh, log1p, expm1 and cbrt of
// the host's C library, whose results are not correctly rounded and differ
// between libraries (the reference's device build uses CUDA's, which differ
// again). Linked into the harness executable, the definitions below take the
// place of the C library's for every call from the reference's objects, so
// the harness runs the reference's own algorithm with correctly rounded
// elementary functions, the ones the GB300 build's FP64 path also uses
// (celeritas_gb300/csrc/gbx/Libm.hh). Any correctly rounded library gives
// the same values, except on the few inputs that Libm.hh documents.
//
// Test infrastructure: linked only into oracle/_ref/ref_harness_pinned.
#include "../../celeritas_gb300/csrc/gbx/Libm.hh"

extern "C"
{
double exp(double x) noexcept
{
    return gbx::libm::exp(x);
}
double log(double x) noexcept
{
    return gbx::libm::log(x);
}
double sin(double x) noexcept
{
    return gbx::libm::sin(x);
}
double cos(double x) noexcept
{
    return gbx::libm::cos(x);
}
void sincos(double x, double* s, double* c) noexcept
{
    *s = gbx::libm::sin(x);
    *c = gbx::libm::cos(x);
}
double tanh(double x) noexcept
{
    return gbx::libm::tanh(x);
}
double log1p(double x) noexcept
{
    return gbx::libm::log1p(x);
}
double expm1(double x) noexcept
{
    return gbx::libm::expm1(x);
}
double cbrt(double x) noexcept
{
    return gbx::libm::cbrt(x);
}
}
