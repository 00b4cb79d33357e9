// Urban multiple scattering: step limitation (safety algorithm), true <->
// geometric path conversion, angular deflection and lateral displacement.
//
// Follows src/celeritas/em/msc/UrbanMsc.hh:97-297 with
// detail/UrbanMscHelper.hh, UrbanMscSafetyStepLimit.hh, MscStepToGeo.hh,
// MscStepFromGeo.hh, UrbanMscScatter.hh and UrbanPositronCorrector.hh, and
// the parameter constants of src/celeritas/em/data/UrbanMscData.hh.
#pragma once

#include "Geometry.hh"
#include "Physics.hh"

namespace gbx
{
namespace msc
{
// UrbanMscParameters
constexpr double nanometer = double(1e-7) * constants::centimeter;
constexpr real_type tau_small = 1e-16;
constexpr real_type tau_big = 8;
constexpr real_type safety_tol = 0.01;
constexpr real_type geom_limit = 5e-8 * constants::millimeter;
constexpr real_type dtrl = 0.05;
constexpr real_type limit_min_fix = real_type(0.01) * nanometer;
constexpr real_type limit_min = 10 * limit_min_fix;
constexpr real_type min_step = 1 * nanometer;
constexpr real_type min_sampling_energy = 1e-6;
constexpr real_type min_scaling_energy = 5e-3;
constexpr real_type small_step_alpha = 0;
}  // namespace msc

//! Helper for per-track msc quantities (UrbanMscHelper)
class MscHelper
{
  public:
    GBX_FORCEINLINE MscHelper(ParamsData const& p,
                              StateData const& s,
                              PhysicsTrack const& phys,
                              size_type slot,
                              size_type particle,
                              size_type material)
        : p_(p), s_(s), phys_(phys), slot_(slot)
    {
        size_type idx = material * 2 + (particle == p.electron_id ? 0 : 1);
        pm_ = p.msc.par_mat + idx;
        xs_ = p.grids + p.ints[p.msc.xs_grids + idx];
        energy_ = s.energy[slot];
        lambda_ = this->calc_msc_mfp(energy_);
    }

    GBX_FORCEINLINE real_type msc_mfp() const { return lambda_; }
    GBX_FORCEINLINE real_type scaled_zeff() const { return pm_->scaled_zeff; }

    GBX_FORCEINLINE real_type calc_msc_mfp(real_type energy) const
    {
        real_type xsec
            = calc_grid_xs(p_, *xs_, energy, phys_.log_energy(energy)) / ipow<2>(energy);
        if constexpr (sizeof(real_type) < sizeof(double))
        {
            // FP32: in a near-vacuum the cross section underflows to zero;
            // a finite mean free path far beyond any step keeps the
            // path conversions finite (tau = step / lambda stays ~0)
            return min_of(1 / xsec, real_type(1e20));
        }
        return 1 / xsec;
    }

    GBX_FORCEINLINE real_type calc_inverse_range(real_type step) const
    {
        XsGrid const* rg = phys_.grid(vgt_range, phys_.group().eloss_process);
        return calc_inverse_range_table(*rg, step);
    }

    GBX_FORCEINLINE real_type max_step() const
    {
        return s_.dedx_range[slot_] * real_type(pm_->d_over_r);
    }

    GBX_FORCEINLINE real_type calc_end_energy(real_type step) const
    {
        real_type range = s_.dedx_range[slot_];
        if (step <= range * msc::dtrl)
        {
            XsGrid const* eg
                = phys_.grid(vgt_energy_loss, phys_.group().eloss_process);
            real_type dedx = calc_grid_xs(p_, *eg, energy_, phys_.log_energy(energy_));
            return energy_ - step * dedx;
        }
        return this->calc_inverse_range(range - step);
    }

  private:
    ParamsData const& p_;
    StateData const& s_;
    PhysicsTrack const& phys_;
    size_type slot_;
    UrbanMscParMatRecord const* pm_;
    XsGrid const* xs_;
    real_type energy_;
    real_type lambda_;

    GBX_FORCEINLINE real_type calc_inverse_range_table(XsGrid const& g,
                                                       real_type r) const
    {
        return ::gbx::calc_inverse_range(p_, g, r);
    }
};

//! Geometric path and slope from a true path (MscStepToGeo)
struct GeoPath
{
    real_type step;
    real_type alpha;
};

GBX_FUNCTION GeoPath msc_true_to_geo(ParamsData const& p,
                                     MscHelper const& helper,
                                     real_type energy,
                                     real_type lambda,
                                     real_type range,
                                     real_type tstep)
{
    GeoPath result;
    result.alpha = msc::small_step_alpha;
    if (tstep < msc::min_step)
    {
        result.step = tstep;
    }
    else if (tstep < range * msc::dtrl)
    {
        result.step = -lambda * libm::expm1(-tstep / lambda);
    }
    else
    {
        real_type mfp_slope;
        real_type const mass = p.particles[p.electron_id].mass;
        if (energy < mass || tstep == range)
        {
            result.alpha = 1 / range;
            mfp_slope = max_of<real_type>(1 - result.alpha * tstep, 0);
        }
        else
        {
            real_type rfinal = range - tstep;
            real_type endpoint_energy = helper.calc_inverse_range(rfinal);
            real_type lambda1 = helper.calc_msc_mfp(endpoint_energy);
            result.alpha = (lambda - lambda1) / (lambda * tstep);
            mfp_slope = lambda1 / lambda;
        }
        real_type w = 1 + 1 / (result.alpha * lambda);
        result.step = (1 - real_type(libm::exp(w * libm::log(mfp_slope))))
                      / (result.alpha * w);
    }
    result.step = min_of(result.step, tstep);
    return result;
}

//! True path from a geometric path (MscStepFromGeo)
GBX_FUNCTION real_type msc_geo_to_true(real_type true_step,
                                       real_type alpha,
                                       real_type range,
                                       real_type lambda,
                                       real_type gstep)
{
    if (gstep < msc::min_step)
    {
        return gstep;
    }
    real_type tstep;
    if (alpha == msc::small_step_alpha)
    {
        tstep = -lambda * libm::log1p(-gstep / lambda);
        if (tstep < msc::min_step)
        {
            tstep = gstep;
        }
    }
    else
    {
        real_type w = 1 + 1 / (alpha * lambda);
        real_type x = alpha * w * gstep;
        x = min_of(x, real_type(1));
        real_type temp = 1 - libm::exp((1 / w) * libm::log(1 - x));
        real_type result = temp / alpha;
        tstep = min_of(result, range);
    }
    // clamp(tstep, gstep, true_step)
    return tstep < gstep ? gstep : (true_step < tstep ? true_step : tstep);
}

GBX_FORCEINLINE real_type msc_displacement(real_type geom_path, real_type true_path)
{
    real_type rmax2 = (true_path - geom_path) * (true_path + geom_path);
    constexpr real_type mean_radius_frac{0.73};
    return mean_radius_frac * std::sqrt(rmax2);
}

//! Whether msc applies to this track for this step (UrbanMsc::is_applicable)
GBX_FORCEINLINE bool msc_is_applicable(ParamsData const& p,
                                       StateData const& s,
                                       size_type slot,
                                       real_type step)
{
    if (!p.msc.enabled)
        return false;
    if (step <= msc::geom_limit)
        return false;
    if (s.status[slot] != status_alive)
        return false;
    size_type pid = s.particle_id[slot];
    if (pid != p.electron_id && pid != p.positron_id)
        return false;
    real_type e = s.energy[slot];
    return e > real_type(p.msc.low_energy_limit)
           && e < real_type(p.msc.high_energy_limit);
}

//! Limit the step due to multiple scattering (MscStepLimitApplier). Returns
//! the FP64 safety distance at the track's position if the limit computed
//! it (0 otherwise), which the field propagation reuses.
template<class G>
GBX_FUNCTION double msc_limit_step(ParamsData const& p,
                                   StateData const& s,
                                   size_type slot,
                                   G& rng)
{
    if (!msc_is_applicable(p, s, slot, s.step_length[slot]))
    {
        s.msc_geom_path[slot] = 0;
        return 0;
    }
    // FP64 safety distance at the step's start when the limit needs it
    double start_safety = 0;
    size_type const pid = s.particle_id[slot];
    size_type const mid = s.material[slot];
    real_type const energy = s.energy[slot];
    PhysicsTrack phys(p, pid, mid, s, slot);
    MscHelper helper(p, s, phys, slot, pid, mid);
    GeoTrackView geo(p.geo, s, slot);
    bool displaced = false;
    real_type const phys_step = s.step_length[slot];

    real_type true_path;
    if (phys_step <= msc::limit_min_fix)
    {
        true_path = phys_step;
    }
    else
    {
        real_type safety = 0;
        bool safe_return = false;
        bool const on_boundary = geo.is_on_boundary();
        if (!on_boundary)
        {
            real_type const max_step = helper.max_step();
            start_safety = geo.find_safety();
            safety = start_safety;
            if (safety >= max_step)
            {
                true_path = phys_step;
                safe_return = true;
            }
        }
        if (!safe_return)
        {
            displaced = true;
            // UrbanMscSafetyStepLimit
            real_type max_step = phys_step;
            real_type const range = s.dedx_range[slot];
            bool const has_range = s.msc_range_init[slot] > 0
                                   && s.msc_range_factor[slot] > 0
                                   && s.msc_limit_min[slot] > 0;
            if (!has_range || on_boundary)
            {
                real_type range_factor = real_type(p.msc.range_factor);
                real_type range_init = max_of<real_type>(range, helper.msc_mfp());
                real_type const lambda_limit = p.msc.lambda_limit;
                if (helper.msc_mfp() > lambda_limit)
                {
                    real_type c = 0.75;
                    range_factor *= c + (1 - c) * helper.msc_mfp() / lambda_limit;
                }
                // calc_limit_min
                UrbanMscMaterialRecord const& md = p.msc.material[mid];
                real_type const cq[3] = {2, real_type(md.stepmin_coeff[0]),
                                         real_type(md.stepmin_coeff[1])};
                real_type xm = helper.msc_mfp() / poly_eval<2>(cq, energy);
                xm *= helper.scaled_zeff();
                if (energy < msc::min_scaling_energy)
                {
                    xm *= (real_type(0.5)
                           + real_type(0.5) * energy / msc::min_scaling_energy);
                }
                real_type limit_min = max_of<real_type>(xm, msc::limit_min_fix);
                s.msc_range_init[slot] = range_init;
                s.msc_range_factor[slot] = range_factor;
                s.msc_limit_min[slot] = limit_min;
            }
            real_type const limit_min = s.msc_limit_min[slot];
            real_type limit = range;
            if (safety < range)
            {
                limit = max_of<real_type>(
                    s.msc_range_factor[slot] * s.msc_range_init[slot],
                    real_type(p.msc.safety_factor) * safety);
            }
            limit = max_of<real_type>(limit, limit_min);
            if (max_step <= limit)
            {
                true_path = max_step;
            }
            else if (limit == limit_min)
            {
                true_path = limit_min;
            }
            else
            {
                NormalDistribution<real_type> sample_gauss(
                    limit, real_type(0.1) * (limit - limit_min));
                real_type sampled = sample_gauss(rng);
                true_path = sampled < limit_min
                                ? limit_min
                                : (max_step < sampled ? max_step : sampled);
            }
        }
    }

    bool limited = (true_path < phys_step);
    GeoPath gp = msc_true_to_geo(
        p, helper, energy, helper.msc_mfp(), s.dedx_range[slot], true_path);
    if (gp.step > helper.msc_mfp())
    {
        gp.step = helper.msc_mfp();
        limited = true;
    }
    s.msc_displaced[slot] = displaced;
    s.msc_true_path[slot] = true_path;
    s.msc_geom_path[slot] = gp.step;
    s.msc_alpha[slot] = gp.alpha;
    s.step_length[slot] = gp.step;
    if (limited)
    {
        s.post_step_action[slot] = p.action_msc_range;
    }
    return start_safety;
}

//! Urban positron correction to the scattering angle width
GBX_FORCEINLINE real_type urban_positron_correction(real_type zeff, real_type y)
{
    real_type const c_a[2] = {real_type(0.994), real_type(-4.08e-3)};
    real_type const c_b[3] = {real_type(7.16), real_type(52.6), real_type(365)};
    real_type const c_c[2] = {real_type(1), real_type(-4.47e-3)};
    real_type const c_m[3]
        = {real_type(1.41125), real_type(-1.86427e-2), real_type(1.84035e-4)};
    real_type const a = poly_eval<1>(c_a, zeff);
    real_type const b = poly_eval<2>(c_b, 1 / zeff);
    real_type const c = poly_eval<1>(c_c, zeff);
    real_type const d = real_type(1.21e-3) * zeff;
    real_type const mult = poly_eval<2>(c_m, zeff);
    constexpr real_type xl = 0.6;
    constexpr real_type xh = 0.9;
    constexpr real_type e = 113;
    real_type x = std::sqrt(y * (y + 2) / ipow<2>(y + 1));
    real_type corr;
    if (x < xl)
    {
        corr = a * (1 - libm::exp(-b * x));
    }
    else if (x > xh)
    {
        corr = c + d * libm::exp(e * (x - 1));
    }
    else
    {
        real_type yl = a * (1 - libm::exp(-b * xl));
        real_type yh = c + d * libm::exp(e * (xh - 1));
        real_type y0 = (yh - yl) / (xh - xl);
        real_type y1 = yl - y0 * xl;
        corr = y0 * x + y1;
    }
    return corr * mult;
}

//! Apply the msc deflection and displacement (MscApplier)
template<class G>
GBX_FUNCTION void msc_apply_step(ParamsData const& p,
                                 StateData const& s,
                                 size_type slot,
                                 G& rng)
{
    if (s.status[slot] != status_alive)
        return;
    if (!(s.msc_geom_path[slot] > 0))
        return;
    size_type const pid = s.particle_id[slot];
    size_type const mid = s.material[slot];
    PhysicsTrack phys(p, pid, mid, s, slot);
    MscHelper helper(p, s, phys, slot, pid, mid);
    GeoTrackView geo(p.geo, s, slot);
    MaterialRecord const& mat = p.materials[mid];

    bool is_displaced = s.msc_displaced[slot];
    real_type true_path = s.msc_true_path[slot];
    real_type geom_path = s.msc_geom_path[slot];
    size_type const post = s.post_step_action[slot];
    if (post == p.action_boundary || post == p.action_propagation_limit)
    {
        geom_path = s.step_length[slot];
        true_path = msc_geo_to_true(true_path,
                                    s.msc_alpha[slot],
                                    s.dedx_range[slot],
                                    helper.msc_mfp(),
                                    geom_path);
        is_displaced = false;
    }
    s.step_length[slot] = true_path;

    real_type safety = 0;
    if (is_displaced)
    {
        real_type displ = msc_displacement(geom_path, true_path);
        displ = max_of(displ * (1 + 2 * msc::safety_tol), msc::geom_limit);
        safety = geo.find_safety();
        if (safety == 0)
        {
            is_displaced = false;
        }
    }

    // UrbanMscScatter
    real_type const inc_energy = s.energy[slot];
    bool const is_positron = (pid == p.positron_id);
    Real3 const inc_dir_d = geo.dir();
    RVec3 const inc_dir{real_type(inc_dir_d.x), real_type(inc_dir_d.y),
                        real_type(inc_dir_d.z)};
    real_type limit_min = s.msc_limit_min[slot];
    real_type end_energy = 0;
    real_type tau = 0, xmean = 0, x2mean = 0, theta0 = -1;
    bool skip_sampling;
    if (true_path == s.dedx_range[slot])
    {
        skip_sampling = true;
    }
    else if (true_path < msc::geom_limit)
    {
        skip_sampling = true;
    }
    else
    {
        end_energy = helper.calc_end_energy(true_path);
        if (end_energy < msc::min_sampling_energy)
            skip_sampling = true;
        else if (true_path <= helper.msc_mfp() * msc::tau_small)
            skip_sampling = true;
        else
            skip_sampling = false;
    }
    UrbanMscMaterialRecord const& md = p.msc.material[mid];
    if (!skip_sampling)
    {
        real_type lambda = helper.msc_mfp();
        real_type lambda_end = helper.calc_msc_mfp(end_energy);
        real_type denom;
        if (std::fabs(lambda - lambda_end) < lambda * real_type(0.01))
            denom = helper.msc_mfp();
        else
            denom = (lambda - lambda_end) / libm::log(lambda / lambda_end);
        tau = true_path / denom;
        if (tau < msc::tau_big)
        {
            xmean = libm::exp(-tau);
            x2mean = (1 + 2 * libm::exp(real_type(-2.5) * tau)) / 3;
            if (limit_min == 0)
                limit_min = msc::limit_min;
            limit_min = min_of(limit_min, real_type(p.msc.lambda_limit));
            // compute_theta0
            real_type const mass = p.particles[p.electron_id].mass;
            real_type tp = max_of(limit_min, true_path);
            real_type y = tp / real_type(mat.rad_length);
            if (is_positron)
            {
                y *= urban_positron_correction(
                    real_type(mat.zeff), std::sqrt(inc_energy * end_energy) / mass);
            }
            real_type invbetacp = std::sqrt(
                (inc_energy + mass) * (end_energy + mass)
                / (inc_energy * (inc_energy + 2 * mass) * end_energy
                   * (end_energy + 2 * mass)));
            constexpr real_type c_highland = 13.6;
            real_type th = c_highland * std::sqrt(y) * invbetacp;
            real_type const tc[2] = {real_type(md.theta_coeff[0]),
                                     real_type(md.theta_coeff[1])};
            th *= poly_eval<1>(tc, libm::log(y));
            if (true_path < limit_min)
            {
                th *= std::sqrt(true_path / limit_min);
            }
            theta0 = max_of<real_type>(th, 0);
            if (theta0 < real_type(1e-8))
            {
                if (!is_displaced)
                    skip_sampling = true;
                else
                    theta0 = 0;
            }
        }
    }
    if (skip_sampling)
        return;

    auto simple_scattering = [&]() -> real_type {
        real_type a = (2 * xmean + 9 * x2mean - 3) / (2 * xmean - 3 * x2mean + 1);
        real_type p_pow = (a + 2) * xmean / a;
        real_type result{};
        do
        {
            real_type rdm = generate_canonical<real_type>(rng);
            result = 2
                         * (sample_bernoulli<real_type>(p_pow, rng)
                                ? real_type(libm::exp((1 / (a + 1)) * libm::log(rdm)))
                                : rdm)
                     - 1;
        } while (std::fabs(result) > 1);
        return result;
    };

    real_type costheta;
    if (theta0 <= 0)
    {
        costheta = 1;
    }
    else if (tau >= msc::tau_big)
    {
        costheta = UniformRealDistribution<real_type>(-1, 1)(rng);
    }
    else if (2 * end_energy < inc_energy || theta0 > real_type(constants::pi / 6))
    {
        costheta = simple_scattering();
    }
    else
    {
        // sample_cos_theta
        real_type maxtau = true_path < limit_min ? limit_min / helper.msc_mfp() : tau;
        real_type u = libm::exp((1 / real_type(6)) * libm::log(maxtau));
        real_type radlen_mfp = true_path / (tau * real_type(mat.rad_length));
        real_type const tq[3] = {real_type(md.tail_coeff[0]),
                                 real_type(md.tail_coeff[1]),
                                 real_type(md.tail_coeff[2])};
        real_type xsi = poly_eval<2>(tq, u)
                        + real_type(md.tail_corr) * libm::log(radlen_mfp);
        xsi = max_of(xsi, real_type(1.9));
        real_type ea = libm::exp(-xsi);
        real_type x = ipow<2>(2 * libm::sin(real_type(0.5) * theta0));
        real_type xmean_1 = 1 - x * (1 + (xsi * ea) / (1 - ea));
        if (xmean_1 <= real_type(0.999) * xmean)
        {
            costheta = simple_scattering();
        }
        else
        {
            real_type c;
            if (std::fabs(xsi - 3) < real_type(0.001))
                c = real_type(3.001);
            else if (std::fabs(xsi - 2) < real_type(0.001))
                c = real_type(2.001);
            else
                c = xsi;
            real_type b1 = 2 + (c - xsi) * x;
            real_type d = libm::exp((c - 1) * libm::log(c * x / b1));
            real_type x0 = 1 - xsi * x;
            real_type xmean_2 = (x0 + d - (c * x - b1 * d) / (c - 2)) / (1 - d);
            real_type f2x0 = (c - 1) / (c * (1 - d));
            real_type prob = f2x0 / (ea / (1 - ea) + f2x0);
            real_type qprob = xmean / (prob * xmean_1 + (1 - prob) * xmean_2);
            if (generate_canonical<real_type>(rng) >= qprob)
            {
                costheta = UniformRealDistribution<real_type>(-1, 1)(rng);
            }
            else if (generate_canonical<real_type>(rng) < prob)
            {
                UniformRealDistribution<real_type> sample_inner(ea, 1);
                costheta = 1 + libm::log(sample_inner(rng)) * x;
            }
            else
            {
                real_type var = (1 - d) * generate_canonical<real_type>(rng);
                if (var < real_type(0.01) * d)
                {
                    var /= (d * (c - 1));
                    costheta = -1
                               + var * (1 - real_type(0.5) * var * c)
                                     * (2 + (c - xsi) * x);
                }
                else
                {
                    costheta = x
                                   * (c - xsi
                                      - c
                                            * real_type(libm::exp(
                                                (-1 / (c - 1)) * libm::log(var + d))))
                               + 1;
                }
            }
        }
    }
    real_type phi = UniformRealDistribution<real_type>(0, 2 * constants::pi)(rng);

    bool displace = false;
    RVec3 displacement{0, 0, 0};
    if (is_displaced)
    {
        real_type length = msc_displacement(geom_path, true_path);
        length = min_of(length, (1 - msc::safety_tol) * safety);
        if (length >= msc::geom_limit)
        {
            // sample_displacement_dir
            constexpr real_type cbeta = 2.160;
            constexpr real_type cbeta1 = 0.9988703417569197;
            real_type psi = -libm::log(1 - generate_canonical<real_type>(rng) * cbeta1)
                            / cbeta;
            real_type dphi = phi;
            dphi += sample_bernoulli<real_type>(real_type(0.5), rng) ? psi : -psi;
            RVec3 dd{libm::cos(dphi), libm::sin(dphi), 0};
            dd = rotate(dd, inc_dir);
            displacement = {dd.x * length, dd.y * length, dd.z * length};
            displace = true;
        }
    }
    RVec3 newdir = rotate(from_spherical(costheta, phi), inc_dir);
    geo.set_dir(to_geo_dir(newdir));
    if (displace)
    {
        Real3 pos = geo.pos();
        geo.move_internal_to(Real3{pos.x + double(displacement.x),
                                   pos.y + double(displacement.y),
                                   pos.z + double(displacement.z)});
    }
}

}  // namespace gbx
