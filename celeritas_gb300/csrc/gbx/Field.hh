// Charged-particle propagation in a uniform magnetic field: Dormand-Prince
// RK5(4) integration with an adaptive driver and a chord-based boundary
// search through the geometry.
//
// Follows src/celeritas/field/FieldPropagator.hh:150-333,
// FieldDriver.hh:182-429, DormandPrinceStepper.hh:102-222,
// MagFieldEquation.hh, detail/FieldUtils.hh and the defaults of
// FieldDriverOptions.hh:26-77.
//
// FP64 build: the whole integration is FP64, operation for operation as in
// the reference. Mixed-precision build: the Runge-Kutta stages (field
// evaluations and stage momenta) are FP32; the positions are accumulated in
// FP64 from FP32 increments; the embedded error vector and the chord
// distance are formed in FP32 from the FP32 stages, and the error norms, the
// acceptance test, the step and the path length are FP64. The step-size
// scale factor err^(-1/5) is FP32.
#pragma once

#include "Geometry.hh"

namespace gbx
{
struct OdeState
{
    Real3 pos;
    Real3 mom;
};

GBX_FORCEINLINE void axpy(double a, OdeState const& x, OdeState* y)
{
    axpy(a, x.pos, &y->pos);
    axpy(a, x.mom, &y->mom);
}

GBX_FORCEINLINE Real3 cross_product(Real3 const& x, Real3 const& y)
{
    return {x.y * y.z - x.z * y.y, x.z * y.x - x.x * y.z, x.x * y.y - x.y * y.x};
}

GBX_FORCEINLINE double fastpow(double a, double b)
{
    return libm::exp(b * libm::log(a));
}

//! Field of an R-Z map at a position (RZMapField::operator(),
//! src/celeritas/field/RZMapField.hh:70-108): bilinear in (r, z) on the
//! uniform grids, zero outside the map, the radial component along (x, y)
GBX_FUNCTION Real3 rzmap_field(RZMapData const& m, Real3 const& pos)
{
    Real3 value{0, 0, 0};
    double const r = std::sqrt(ipow<2>(pos.x) + ipow<2>(pos.y));
    if (!(pos.z >= m.z.front && pos.z <= m.z.back && r >= m.r.front && r <= m.r.back))
        return value;
    // find_interp on a uniform grid (UniformGrid::find, operator[]); a value
    // on the last node takes the last interval
    auto locate = [](FieldMapGrid const& g, double v, size_type* index) {
        size_type i = static_cast<size_type>((v - g.front) / g.delta);
        i = min_of(i, g.size - 2);
        double const lower = g.front + g.delta * i;
        double const upper = g.front + g.delta * (i + 1);
        *index = i;
        return (v - lower) / (upper - lower);
    };
    size_type ir, iz;
    double const fr = locate(m.r, r, &ir);
    double const fz = locate(m.z, pos.z, &iz);
    size_type const nr = m.r.size;
    double low = m.values[iz * nr + ir].value_z;
    double high = m.values[(iz + 1) * nr + ir].value_z;
    value.z = low + (high - low) * fz;
    low = m.values[iz * nr + ir].value_r;
    high = m.values[iz * nr + ir + 1].value_r;
    double const tmp = (r != 0) ? (low + (high - low) * fr) / r : low;
    value.x = tmp * pos.x;
    value.y = tmp * pos.y;
    return value;
}

//! The R-Z map's field in FP32 (the mixed-precision stages): the same
//! interpolation on the FP32 nodes at an FP32 position
GBX_NOINLINE Vec3<float> rzmap_field_f(RZMapData const& m, Vec3<float> const& pos)
{
    Vec3<float> value{0, 0, 0};
    float const r = std::sqrt(pos.x * pos.x + pos.y * pos.y);
    if (!(pos.z >= float(m.z.front) && pos.z <= float(m.z.back) && r >= float(m.r.front)
          && r <= float(m.r.back)))
        return value;
    auto locate = [](FieldMapGrid const& g, float v, size_type* index) {
        float const u = (v - float(g.front)) / float(g.delta);
        size_type const i = min_of(static_cast<size_type>(u), g.size - 2);
        *index = i;
        return u - float(i);
    };
    size_type ir, iz;
    float const fr = locate(m.r, r, &ir);
    float const fz = locate(m.z, pos.z, &iz);
    size_type const nr = m.r.size;
    FieldMapElementF const* v = m.values_f;
    float low = v[iz * nr + ir].value_z;
    float high = v[(iz + 1) * nr + ir].value_z;
    value.z = low + (high - low) * fz;
    low = v[iz * nr + ir].value_r;
    high = v[iz * nr + ir + 1].value_r;
    float const tmp = (r != 0) ? (low + (high - low) * fr) / r : low;
    value.x = tmp * pos.x;
    value.y = tmp * pos.y;
    return value;
}

//! Equation of motion in a magnetic field: d(pos)/ds = p/|p|,
//! d(mom)/ds = (q/|p|) p x B(pos) (MagFieldEquation). The field is uniform,
//! or an R-Z map evaluated at the state's position when 'map' is set.
struct UniformFieldEquation
{
    Real3 field;
    double coeffi;
    RZMapData const* map{nullptr};

    GBX_FORCEINLINE OdeState operator()(OdeState const& y) const
    {
        double momentum_inv = 1.0 / std::sqrt(dot_product(y.mom, y.mom));
        OdeState result;
        result.pos = {momentum_inv * y.mom.x,
                      momentum_inv * y.mom.y,
                      momentum_inv * y.mom.z};
        double const scale = coeffi * momentum_inv;
        Real3 c = cross_product(y.mom, map ? rzmap_field(*map, y.pos) : field);
        result.mom = {scale * c.x, scale * c.y, scale * c.z};
        return result;
    }
};

struct FieldStepperResult
{
    OdeState mid_state;  //!< FP64 build only
    OdeState end_state;
    OdeState err_state;  //!< FP64 build only
    // Mixed-precision build only: the embedded error estimate and the chord
    // distance, formed in FP32 from the FP32 stages
    Vec3<float> err_pos_rate;  //!< position error / step = sum_i d_i k_pos_i
    Vec3<float> err_mom;  //!< momentum error = step * sum_i d_i k_mom_i
    float dchord;  //!< sagitta of the midpoint from the chord
};

//! The field equation with its field source fixed at compile time, so that
//! each FP64 Runge-Kutta step branches once on the source, not per stage
template<bool UseMap>
struct FixedFieldEquation
{
    UniformFieldEquation const& eq;

    GBX_FORCEINLINE OdeState operator()(OdeState const& y) const
    {
        double momentum_inv = 1.0 / std::sqrt(dot_product(y.mom, y.mom));
        OdeState result;
        result.pos = {momentum_inv * y.mom.x,
                      momentum_inv * y.mom.y,
                      momentum_inv * y.mom.z};
        double const scale = eq.coeffi * momentum_inv;
        Real3 c = cross_product(y.mom, UseMap ? rzmap_field(*eq.map, y.pos) : eq.field);
        result.mom = {scale * c.x, scale * c.y, scale * c.z};
        return result;
    }
};

//! Dormand-Prince 5(4) step with Shampine's midpoint interpolation
template<class Equation>
GBX_FUNCTION FieldStepperResult dormand_prince_step_fp64(Equation const& rhs,
                                                         double step,
                                                         OdeState const& beg_state)
{
    using R = double;
    constexpr R a11 = 0.2;
    constexpr R a21 = 0.075;
    constexpr R a22 = 0.225;
    constexpr R a31 = 44 / R(45);
    constexpr R a32 = -56 / R(15);
    constexpr R a33 = 32 / R(9);
    constexpr R a41 = 19372 / R(6561);
    constexpr R a42 = -25360 / R(2187);
    constexpr R a43 = 64448 / R(6561);
    constexpr R a44 = -212 / R(729);
    constexpr R a51 = 9017 / R(3168);
    constexpr R a52 = -355 / R(33);
    constexpr R a53 = 46732 / R(5247);
    constexpr R a54 = 49 / R(176);
    constexpr R a55 = -5103 / R(18656);
    constexpr R a61 = 35 / R(384);
    constexpr R a63 = 500 / R(1113);
    constexpr R a64 = 125 / R(192);
    constexpr R a65 = -2187 / R(6784);
    constexpr R a66 = 11 / R(84);
    constexpr R d71 = a61 - 5179 / R(57600);
    constexpr R d73 = a63 - 7571 / R(16695);
    constexpr R d74 = a64 - 393 / R(640);
    constexpr R d75 = a65 + 92097 / R(339200);
    constexpr R d76 = a66 - 187 / R(2100);
    constexpr R d77 = -1 / R(40);
    constexpr R c71 = R(6025192743.) / R(30085553152.);
    constexpr R c73 = R(51252292925.) / R(65400821598.);
    constexpr R c74 = R(-2691868925.) / R(45128329728.);
    constexpr R c75 = R(187940372067.) / R(1594534317056.);
    constexpr R c76 = R(-1776094331.) / R(19743644256.);
    constexpr R c77 = R(11237099.) / R(235043384.);

    FieldStepperResult result;
    OdeState k1 = rhs(beg_state);
    OdeState state = beg_state;
    axpy(a11 * step, k1, &state);
    OdeState k2 = rhs(state);
    state = beg_state;
    axpy(a21 * step, k1, &state);
    axpy(a22 * step, k2, &state);
    OdeState k3 = rhs(state);
    state = beg_state;
    axpy(a31 * step, k1, &state);
    axpy(a32 * step, k2, &state);
    axpy(a33 * step, k3, &state);
    OdeState k4 = rhs(state);
    state = beg_state;
    axpy(a41 * step, k1, &state);
    axpy(a42 * step, k2, &state);
    axpy(a43 * step, k3, &state);
    axpy(a44 * step, k4, &state);
    OdeState k5 = rhs(state);
    state = beg_state;
    axpy(a51 * step, k1, &state);
    axpy(a52 * step, k2, &state);
    axpy(a53 * step, k3, &state);
    axpy(a54 * step, k4, &state);
    axpy(a55 * step, k5, &state);
    OdeState k6 = rhs(state);
    result.end_state = beg_state;
    axpy(a61 * step, k1, &result.end_state);
    axpy(a63 * step, k3, &result.end_state);
    axpy(a64 * step, k4, &result.end_state);
    axpy(a65 * step, k5, &result.end_state);
    axpy(a66 * step, k6, &result.end_state);
    OdeState k7 = rhs(result.end_state);
    result.err_state = {{0, 0, 0}, {0, 0, 0}};
    axpy(d71 * step, k1, &result.err_state);
    axpy(d73 * step, k3, &result.err_state);
    axpy(d74 * step, k4, &result.err_state);
    axpy(d75 * step, k5, &result.err_state);
    axpy(d76 * step, k6, &result.err_state);
    axpy(d77 * step, k7, &result.err_state);
    double half_step = step / double(2);
    result.mid_state = beg_state;
    axpy(c71 * half_step, k1, &result.mid_state);
    axpy(c73 * half_step, k3, &result.mid_state);
    axpy(c74 * half_step, k4, &result.mid_state);
    axpy(c75 * half_step, k5, &result.mid_state);
    axpy(c76 * half_step, k6, &result.mid_state);
    axpy(c77 * half_step, k7, &result.mid_state);
    return result;
}


//! Mixed-precision Dormand-Prince 5(4) step. The stages carry FP32 momenta,
//! FP32 derivatives and, for a field map, FP32 position increments from the
//! start at which the map is read in FP32; the end position is the FP64
//! start plus an FP32 increment. The embedded error estimate (a weighted sum
//! of the FP32 stage derivatives) and the chord distance (from the FP32
//! increments to the end and to Shampine's midpoint) are formed in FP32:
//! their inputs carry FP32 rounding, which FP64 arithmetic on them would not
//! remove. The field driver takes the error norms and the acceptance test in FP64.
GBX_FUNCTION FieldStepperResult dormand_prince_step_mixed(UniformFieldEquation const& rhs,
                                                          double step,
                                                          OdeState const& beg_state)
{
    using F = float;
    using F3 = Vec3<float>;
    // Butcher tableau of the FP64 stepper, rounded to FP32
    constexpr F a11 = 0.2f;
    constexpr F a21 = 0.075f, a22 = 0.225f;
    constexpr F a31 = F(44. / 45), a32 = F(-56. / 15), a33 = F(32. / 9);
    constexpr F a41 = F(19372. / 6561), a42 = F(-25360. / 2187),
                a43 = F(64448. / 6561), a44 = F(-212. / 729);
    constexpr F a51 = F(9017. / 3168), a52 = F(-355. / 33), a53 = F(46732. / 5247),
                a54 = F(49. / 176), a55 = F(-5103. / 18656);
    constexpr double b1 = 35. / 384, b3 = 500. / 1113, b4 = 125. / 192,
                     b5 = -2187. / 6784, b6 = 11. / 84;
    constexpr double d1 = b1 - 5179. / 57600, d3 = b3 - 7571. / 16695,
                     d4 = b4 - 393. / 640, d5 = b5 + 92097. / 339200,
                     d6 = b6 - 187. / 2100, d7 = -1. / 40;
    constexpr F c1 = F(6025192743. / 30085553152.), c3 = F(51252292925. / 65400821598.),
                c4 = F(-2691868925. / 45128329728.),
                c5 = F(187940372067. / 1594534317056.),
                c6 = F(-1776094331. / 19743644256.), c7 = F(11237099. / 235043384.);

    F3 const uniform{F(rhs.field.x), F(rhs.field.y), F(rhs.field.z)};
    F const coeffi = F(rhs.coeffi);
    // Start position in FP32, for field-map lookups only
    F3 const p0{F(beg_state.pos.x), F(beg_state.pos.y), F(beg_state.pos.z)};
    // d(pos)/ds = p/|p|, d(mom)/ds = (q/|p|) p x B(pos), at the stage's
    // position increment 'dp' from the start
    auto eval = [&](F3 const& dp, F3 const& m, F3* kpos, F3* kmom) {
        F3 const field
            = rhs.map ? rzmap_field_f(*rhs.map, F3{p0.x + dp.x, p0.y + dp.y, p0.z + dp.z})
                      : uniform;
        F const inv = F(1) / std::sqrt(m.x * m.x + m.y * m.y + m.z * m.z);
        *kpos = {m.x * inv, m.y * inv, m.z * inv};
        F const scale = coeffi * inv;
        *kmom = {scale * (m.y * field.z - m.z * field.y),
                 scale * (m.z * field.x - m.x * field.z),
                 scale * (m.x * field.y - m.y * field.x)};
    };
    // Stage momentum m0 + h * sum_j a[j] k_mom[j]
    auto stage = [](F3 const& m0, F h, F const* a, int n, F3 const* k) {
        F3 r = m0;
#pragma unroll
        for (int j = 0; j < n; ++j)
        {
            r.x += h * a[j] * k[j].x;
            r.y += h * a[j] * k[j].y;
            r.z += h * a[j] * k[j].z;
        }
        return r;
    };
    F const A1[1] = {a11};
    F const A2[2] = {a21, a22};
    F const A3[3] = {a31, a32, a33};
    F const A4[4] = {a41, a42, a43, a44};
    F const A5[5] = {a51, a52, a53, a54, a55};

    F const h = F(step);
    F3 const m0{F(beg_state.mom.x), F(beg_state.mom.y), F(beg_state.mom.z)};
    F3 const zero{0, 0, 0};
    F3 kp[7], km[7];
    // Stage position increments matter only for a field map
    auto dpos_at = [&](F const* a, int n) {
        return rhs.map ? stage(zero, h, a, n, kp) : zero;
    };
    eval(zero, m0, &kp[0], &km[0]);
    eval(dpos_at(A1, 1), stage(m0, h, A1, 1, km), &kp[1], &km[1]);
    eval(dpos_at(A2, 2), stage(m0, h, A2, 2, km), &kp[2], &km[2]);
    eval(dpos_at(A3, 3), stage(m0, h, A3, 3, km), &kp[3], &km[3]);
    eval(dpos_at(A4, 4), stage(m0, h, A4, 4, km), &kp[4], &km[4]);
    eval(dpos_at(A5, 5), stage(m0, h, A5, 5, km), &kp[5], &km[5]);
    // Fifth-order solution: FP32 increments added to the FP64 start
    F const bf[7] = {F(b1), 0, F(b3), F(b4), F(b5), F(b6), 0};
    F3 dpos{0, 0, 0}, m_end = m0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        dpos.x += bf[i] * kp[i].x;
        dpos.y += bf[i] * kp[i].y;
        dpos.z += bf[i] * kp[i].z;
        m_end.x += h * bf[i] * km[i].x;
        m_end.y += h * bf[i] * km[i].y;
        m_end.z += h * bf[i] * km[i].z;
    }
    F3 const end_inc{h * dpos.x, h * dpos.y, h * dpos.z};
    eval(end_inc, m_end, &kp[6], &km[6]);

    FieldStepperResult result;
    result.end_state.pos = {beg_state.pos.x + double(end_inc.x),
                            beg_state.pos.y + double(end_inc.y),
                            beg_state.pos.z + double(end_inc.z)};
    result.end_state.mom = {double(m_end.x), double(m_end.y), double(m_end.z)};

    // Embedded error estimate: difference of the fifth- and fourth-order
    // solutions, sum_i d_i k_i (times the step for the momentum)
    F const df[7] = {F(d1), 0, F(d3), F(d4), F(d5), F(d6), F(d7)};
    F3 epos{0, 0, 0}, emom{0, 0, 0};
#pragma unroll
    for (int i = 0; i < 7; ++i)
    {
        if (i == 1)
            continue;
        epos.x += df[i] * kp[i].x;
        epos.y += df[i] * kp[i].y;
        epos.z += df[i] * kp[i].z;
        emom.x += df[i] * km[i].x;
        emom.y += df[i] * km[i].y;
        emom.z += df[i] * km[i].z;
    }
    result.err_pos_rate = epos;
    result.err_mom = {h * emom.x, h * emom.y, h * emom.z};

    // Shampine midpoint increment, and its distance from the chord
    F const cf[7] = {c1, 0, c3, c4, c5, c6, c7};
    F3 mpos{0, 0, 0};
#pragma unroll
    for (int i = 0; i < 7; ++i)
    {
        mpos.x += cf[i] * kp[i].x;
        mpos.y += cf[i] * kp[i].y;
        mpos.z += cf[i] * kp[i].z;
    }
    F const half = F(0.5) * h;
    F3 const mid_inc{half * mpos.x, half * mpos.y, half * mpos.z};
    F3 const cr{end_inc.y * mid_inc.z - end_inc.z * mid_inc.y,
                end_inc.z * mid_inc.x - end_inc.x * mid_inc.z,
                end_inc.x * mid_inc.y - end_inc.y * mid_inc.x};
    result.dchord = std::sqrt((cr.x * cr.x + cr.y * cr.y + cr.z * cr.z)
                              / (end_inc.x * end_inc.x + end_inc.y * end_inc.y
                                 + end_inc.z * end_inc.z));
    return result;
}

//! Dormand-Prince step of this build's precision
GBX_FORCEINLINE FieldStepperResult dormand_prince_step(UniformFieldEquation const& rhs,
                                                       double step,
                                                       OdeState const& beg_state)
{
    if constexpr (sizeof(real_type) == sizeof(double))
    {
        if (rhs.map)
            return dormand_prince_step_fp64(FixedFieldEquation<true>{rhs}, step, beg_state);
        return dormand_prince_step_fp64(FixedFieldEquation<false>{rhs}, step, beg_state);
    }
    else
    {
        return dormand_prince_step_mixed(rhs, step, beg_state);
    }
}

//---------------------------------------------------------------------------//
// Field driver
//---------------------------------------------------------------------------//
struct DriverResult
{
    OdeState state;
    double step;
};

class FieldDriver
{
  public:
    GBX_FORCEINLINE FieldDriver(FieldOptions const& options,
                                UniformFieldEquation const& rhs)
        : opt_(options), rhs_(rhs)
    {
    }

    GBX_FUNCTION DriverResult advance(double step, OdeState const& state)
    {
        if (step <= opt_.minimum_step)
        {
            DriverResult result;
            result.state = dormand_prince_step(rhs_, step, state).end_state;
            result.step = step;
            return result;
        }
        ChordSearch output = this->find_next_chord(min_of(step, max_chord_), state);
        if (output.end.step < step)
        {
            max_chord_ = output.end.step * (1 / FieldOptions::min_chord_shrink);
        }
        if (output.err_sq > 1)
        {
            double next_step = step * this->new_step_scale(output.err_sq);
            output.end = this->accurate_advance(output.end.step, state, next_step);
        }
        return output.end;
    }

    //! Forget the chord limit of the previous propagation
    GBX_FORCEINLINE void reset() { max_chord_ = INFINITY; }
    GBX_FORCEINLINE void set_rhs(UniformFieldEquation const& rhs) { rhs_ = rhs; }

    GBX_FORCEINLINE double minimum_step() const { return opt_.minimum_step; }
    GBX_FORCEINLINE double delta_intersection() const
    {
        return opt_.delta_intersection;
    }
    GBX_FORCEINLINE short max_substeps() const { return opt_.max_substeps; }

  private:
    struct ChordSearch
    {
        DriverResult end;
        double err_sq;
    };
    struct Integration
    {
        DriverResult end;
        double proposed_step;
    };

    FieldOptions const& opt_;
    UniformFieldEquation rhs_;
    double max_chord_{INFINITY};

    static GBX_FORCEINLINE double rel_err_sq(OdeState const& err_state,
                                             double step,
                                             Real3 const& mom)
    {
        double errpos2 = dot_product(err_state.pos, err_state.pos);
        double errvel2 = dot_product(err_state.mom, err_state.mom);
        errpos2 /= ipow<2>(step);
        errvel2 /= dot_product(mom, mom);
        return max_of(errpos2, errvel2);
    }

    //! Scaled error of a stepper result: above 1 the step is rejected
    GBX_FORCEINLINE double step_err_sq(FieldStepperResult const& result,
                                       double step,
                                       Real3 const& mom) const
    {
        if constexpr (sizeof(real_type) == sizeof(double))
        {
            return rel_err_sq(result.err_state, step, mom)
                   / ipow<2>(opt_.epsilon_rel_max);
        }
        else
        {
            // FP64 norms of the FP32 error estimate; the position error
            // comes as a rate, so no division by the step is needed
            Real3 const ep{double(result.err_pos_rate.x),
                           double(result.err_pos_rate.y),
                           double(result.err_pos_rate.z)};
            Real3 const em{double(result.err_mom.x),
                           double(result.err_mom.y),
                           double(result.err_mom.z)};
            double const errpos2 = dot_product(ep, ep);
            double const errvel2 = dot_product(em, em) / dot_product(mom, mom);
            return max_of(errpos2, errvel2) / ipow<2>(opt_.epsilon_rel_max);
        }
    }

    //! Distance of the stepper's midpoint from the chord
    GBX_FORCEINLINE double chord_distance(FieldStepperResult const& result,
                                          OdeState const& state) const
    {
        if constexpr (sizeof(real_type) == sizeof(double))
            return distance_chord(state.pos, result.mid_state.pos, result.end_state.pos);
        else
            return double(result.dchord);
    }

    static GBX_FORCEINLINE double distance_chord(Real3 const& beg_pos,
                                                 Real3 const& mid_pos,
                                                 Real3 const& end_pos)
    {
        Real3 beg_mid{mid_pos.x - beg_pos.x, mid_pos.y - beg_pos.y, mid_pos.z - beg_pos.z};
        Real3 beg_end{end_pos.x - beg_pos.x, end_pos.y - beg_pos.y, end_pos.z - beg_pos.z};
        Real3 cross = cross_product(beg_end, beg_mid);
        return std::sqrt(dot_product(cross, cross) / dot_product(beg_end, beg_end));
    }

    GBX_FORCEINLINE double new_step_scale(double err_sq) const
    {
        double const power = 0.5 * (err_sq > 1 ? opt_.pshrink : opt_.pgrow);
        if constexpr (sizeof(real_type) == sizeof(double))
        {
            return opt_.safety * fastpow(err_sq, power);
        }
        else
        {
            // Heuristic step-size factor in FP32 (the acceptance test that
            // uses err_sq stays FP64); clamp the argument to FP32 range
            float const e = float(min_of(max_of(err_sq, 1e-30), 1e30));
            return opt_.safety * double(libm::exp(float(power) * libm::log(e)));
        }
    }

    GBX_FUNCTION ChordSearch find_next_chord(double step, OdeState const& state) const
    {
        ChordSearch output;
        bool succeeded = false;
        auto remaining_steps = opt_.max_nsteps;
        FieldStepperResult result;
        do
        {
            result = dormand_prince_step(rhs_, step, state);
            double dchord = this->chord_distance(result, state);
            if (dchord > opt_.delta_chord + FieldOptions::dchord_tol)
            {
                double scale_step = max_of(std::sqrt(opt_.delta_chord / dchord),
                                           FieldOptions::min_chord_shrink);
                step *= scale_step;
            }
            else
            {
                succeeded = true;
            }
        } while (!succeeded && --remaining_steps > 0);
        output.end.step = step;
        output.end.state = result.end_state;
        output.err_sq = this->step_err_sq(result, step, state.mom);
        return output;
    }

    GBX_FUNCTION Integration one_good_step(double step, OdeState const& state) const
    {
        Integration output;
        bool succeeded = false;
        size_type remaining_steps = opt_.max_nsteps;
        double err_sq;
        FieldStepperResult result;
        do
        {
            result = dormand_prince_step(rhs_, step, state);
            err_sq = this->step_err_sq(result, step, state.mom);
            if (err_sq > 1)
            {
                step *= max_of(this->new_step_scale(err_sq),
                               opt_.max_stepping_decrease);
            }
            else
            {
                succeeded = true;
            }
        } while (!succeeded && --remaining_steps > 0);
        output.end.state = result.end_state;
        output.end.step = step;
        output.proposed_step
            = step * min_of(this->new_step_scale(err_sq), opt_.max_stepping_increase);
        return output;
    }

    GBX_FUNCTION Integration integrate_step(double step, OdeState const& state) const
    {
        Integration output;
        if (step > opt_.minimum_step)
        {
            output = this->one_good_step(step, state);
        }
        else
        {
            FieldStepperResult result = dormand_prince_step(rhs_, step, state);
            output.end.state = result.end_state;
            output.end.step = step;
            double err_sq = this->step_err_sq(result, step, state.mom);
            output.proposed_step = step * this->new_step_scale(err_sq);
        }
        return output;
    }

    GBX_FUNCTION DriverResult accurate_advance(double step,
                                               OdeState const& state,
                                               double hinitial) const
    {
        double end_curve_length = step;
        double h = ((hinitial > FieldOptions::initial_step_tol * step)
                    && (hinitial < step))
                       ? hinitial
                       : step;
        double h_threshold = opt_.epsilon_step * step;
        Integration output;
        output.end.state = state;
        bool succeeded = false;
        double curve_length = 0;
        auto remaining_steps = opt_.max_nsteps;
        do
        {
            output = this->integrate_step(h, output.end.state);
            curve_length += output.end.step;
            if (h < h_threshold || curve_length >= end_curve_length)
            {
                succeeded = true;
            }
            else
            {
                h = min_of(max_of(output.proposed_step, opt_.minimum_step),
                           end_curve_length - curve_length);
            }
        } while (!succeeded && --remaining_steps > 0);
        output.end.step = min_of(curve_length, step);
        return output.end;
    }
};

//---------------------------------------------------------------------------//
// Field propagator
//---------------------------------------------------------------------------//
#ifdef GBX_CHECK_SAFE_BALL
//! Chord queries the surface-free ball answered, and those the full query
//! contradicted (CPU oracle check build only, single-threaded runs)
inline unsigned long long safe_ball_uses = 0;
inline unsigned long long safe_ball_mismatches = 0;
#endif

//! Propagation of a charged track up to 'step' along its curved trajectory,
//! stopping at the first boundary crossing (FieldPropagator::operator()),
//! split into its set-up, one substep of its loop and its completion so that
//! a kernel can interleave the substeps of different tracks. Running
//! init(), then substep() until done(), then finish() is the reference's
//! sequence of operations.
class FieldPropagation
{
  public:
    GBX_FORCEINLINE FieldPropagation(FieldOptions const& opt,
                                     UniformFieldEquation const& rhs)
        : driver_(opt, rhs)
    {
    }

    //! Start a propagation; 'start_safety' is a safety distance already
    //! known at the track's position (0 if none)
    GBX_FORCEINLINE void
    init(GeoTrackView& geo, double momentum, double step, double start_safety = 0)
    {
        driver_.reset();
        state_.pos = geo.pos();
        Real3 const dir0 = geo.dir();
        state_.mom = {momentum * dir0.x, momentum * dir0.y, momentum * dir0.z};
        result_ = {0, geo.is_on_boundary(), false};
        safe_radius_ = 0;
        if (start_safety > 0 && off_axis(state_.pos))
        {
            double const radius = start_safety * (1 - 1e-6) - 1e-6;
            if (radius > 0)
            {
                safe_radius_ = radius;
                center_ = state_.pos;
            }
        }
        step_ = step;
        remaining_ = step;
        remaining_substeps_ = driver_.max_substeps();
    }

    //! Whether the substep loop has ended (checked after each substep)
    GBX_FORCEINLINE bool done() const
    {
        return !(remaining_ > driver_.minimum_step() && remaining_substeps_ > 0);
    }

    //! One iteration of the substep loop
    GBX_FUNCTION void substep(GeoTrackView& geo)
    {
        double const delta_intersection = driver_.delta_intersection();
        double const minimum_substep = driver_.minimum_step();
        double const bump_distance = delta_intersection * double(0.1);

        DriverResult substep = driver_.advance(remaining_, state_);
        // Chord from the current position to the substep end
        Real3 cdir{substep.state.pos.x - state_.pos.x,
                   substep.state.pos.y - state_.pos.y,
                   substep.state.pos.z - state_.pos.z};
        double const clen = norm(cdir);
        if constexpr (sizeof(real_type) == sizeof(double))
        {
            cdir.x /= clen;
            cdir.y /= clen;
            cdir.z /= clen;
        }
        else
        {
            // One FP64 division instead of three
            double const inv_clen = 1 / clen;
            cdir.x *= inv_clen;
            cdir.y *= inv_clen;
            cdir.z *= inv_clen;
        }
        // The geometry's direction is always the last chord's (a query of a
        // later substep with a chord shorter than the minimum uses it)
        if (clen >= minimum_substep)
        {
            geo.set_dir(cdir);
        }
        double const max_dist = clen + delta_intersection;
#ifdef GBX_CHECK_SAFE_BALL
        // CPU oracle check build: always run the full query, and count the
        // queries the ball would have answered and any it would have got
        // wrong
        bool const ball = this->inside_safe_ball(geo, max_dist);
        Propagation linear_step = geo.find_next_step(max_dist);
        if (ball)
        {
            ++safe_ball_uses;
            if (linear_step.boundary || linear_step.distance != max_dist)
                ++safe_ball_mismatches;
        }
#else
        Propagation linear_step = this->inside_safe_ball(geo, max_dist)
                                      ? geo.no_crossing(max_dist)
                                      : geo.find_next_step(max_dist);
#endif
        if (!linear_step.boundary)
        {
            state_ = substep.state;
            result_.boundary = false;
            result_.distance += substep.step;
            remaining_ = step_ - result_.distance;
            geo.move_internal_to(state_.pos);
            --remaining_substeps_;
            return;
        }
        // Scaled length of the chord up to the crossing (only with one)
        double const update_length = substep.step * linear_step.distance / clen;
        auto is_intercept_close = [&]() {
            double delta_sq = 0;
            for (int i = 0; i < 3; ++i)
            {
                delta_sq += ipow<2>(state_.pos[i] - substep.state.pos[i]
                                    + linear_step.distance * cdir[i]);
            }
            return delta_sq <= ipow<2>(delta_intersection);
        };
        if (result_.boundary && (linear_step.distance) < bump_distance)
        {
            remaining_ = substep.step / 2;
        }
        else if (update_length <= minimum_substep || is_intercept_close()
                 || clen == 0)
        {
            result_.boundary = (linear_step.distance <= clen
                                || result_.distance + update_length <= step_
                                || clen == 0);
            if (!result_.boundary)
            {
                state_.pos = substep.state.pos;
                geo.move_internal_to(substep.state.pos);
            }
            result_.distance += min_of(update_length, substep.step);
            state_.mom = substep.state.mom;
            remaining_ = 0;
        }
        else
        {
            remaining_ = update_length;
        }
    }

    //! Complete the propagation after the loop
    GBX_FUNCTION Propagation finish(GeoTrackView& geo)
    {
        double const bump_distance = driver_.delta_intersection() * double(0.1);
        if (remaining_substeps_ == 0 && result_.distance < step_)
        {
            result_.looping = true;
        }
        else if (result_.distance > 0)
        {
            if (result_.boundary)
            {
                geo.move_to_boundary();
                state_.pos = geo.pos();
            }
            else if (result_.distance < step_)
            {
                result_.distance = step_;
            }
        }
        Real3 dir = make_unit_vector(state_.mom);
        geo.set_dir(dir);
        if (result_.distance == 0)
        {
            result_.distance = min_of(bump_distance, step_);
            result_.boundary = false;
            axpy(result_.distance, dir, &state_.pos);
            geo.move_internal_to(state_.pos);
        }
        return result_;
    }

    GBX_FORCEINLINE void set_rhs(UniformFieldEquation const& rhs)
    {
        driver_.set_rhs(rhs);
    }

  private:
    //! Whether the safety distance at a point bounds the distance to every
    //! surface: on (or within 1e-150 of) the z axis a z cylinder's safety is
    //! taken as infinite (its normal is undefined there, as in the
    //! reference's CalcSafetyDistance), so no ball is centred there
    static GBX_FORCEINLINE bool off_axis(Real3 const& pos)
    {
        return ipow<2>(pos.x) + ipow<2>(pos.y) > 1e-300;
    }

    //! Whether the chord query from the current position reaches no
    //! surface within max_dist, because the segment lies inside a ball that
    //! holds no surface of the current volume: then find_next_step would
    //! return max_dist without a crossing, and no_crossing() leaves the
    //! same result and state without solving the surfaces. Without a known
    //! safety the ball is centred where the track stands after its first
    //! substep of the step (a step of one substep never pays for it), with
    //! the safety distance
    //! there as radius, shrunk by 1e-6 relative and 1e-6 cm so that FP64
    //! rounding of the safety and of the distances cannot admit a crossing
    //! the full query would find. Any point of a plane or z cylinder is at
    //! least the safety distance (|x - v|, |r - R|) from the centre. A
    //! safety the multiple-scattering step limit measured at the start
    //! gives the ball from the first substep on.
    GBX_FUNCTION bool inside_safe_ball(GeoTrackView& geo, double max_dist)
    {
        if (safe_radius_ < 0 || !geo.is_clear_of_boundary())
            return false;
        if (safe_radius_ == 0)
        {
            if (result_.distance == 0 || !off_axis(state_.pos))
                return false;
            double const radius = geo.find_safety() * (1 - 1e-6) - 1e-6;
            if (!(radius > 0))
            {
                safe_radius_ = -1;
                return false;
            }
            safe_radius_ = radius;
            center_ = state_.pos;
        }
        double const room = safe_radius_ - max_dist;
        if (!(room > 0))
            return false;
        double dsq = 0;
        for (int i = 0; i < 3; ++i)
            dsq += ipow<2>(state_.pos[i] - center_[i]);
        return dsq < room * room;
    }

  public:

  private:
    FieldDriver driver_;
    OdeState state_;
    Propagation result_;
    //! Ball free of surfaces: its center and radius (0: not yet measured,
    //! negative: too small to use)
    Real3 center_;
    double safe_radius_;
    double step_;
    double remaining_;
    short remaining_substeps_;
};

//! Propagate a charged track up to 'step' along its curved trajectory,
//! stopping at the first boundary crossing (FieldPropagator::operator())
GBX_FUNCTION Propagation propagate_in_field(FieldOptions const& opt,
                                            UniformFieldEquation const& rhs,
                                            double momentum,
                                            GeoTrackView& geo,
                                            double step)
{
    FieldPropagation fp(opt, rhs);
    fp.init(geo, momentum, step);
    do
    {
        fp.substep(geo);
    } while (!fp.done());
    return fp.finish(geo);
}

}  // namespace gbx
