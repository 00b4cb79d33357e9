// Discrete EM interactions: Klein-Nishina Compton scattering, Livermore
// photoelectric effect, Bethe-Heitler pair production, Seltzer-Berger
// bremsstrahlung, Moller/Bhabha ionization and two-photon positron
// annihilation.
//
// Each sampler consumes the per-slot XORWOW stream in exactly the order of
// the corresponding reference interactor so that outputs agree for the same
// RNG state:
//   src/celeritas/em/interactor/KleinNishinaInteractor.hh:104-190
//   src/celeritas/em/interactor/LivermorePEInteractor.hh:145-360
//   src/celeritas/em/interactor/BetheHeitlerInteractor.hh:165-330
//   src/celeritas/em/interactor/SeltzerBergerInteractor.hh:142-180,
//     interactor/detail/SBEnergySampler.hh, distribution/SBEnergyDistHelper.hh,
//     interactor/detail/SBPositronXsCorrector.hh
//   src/celeritas/em/interactor/MollerBhabhaInteractor.hh:119-160,
//     distribution/MollerEnergyDistribution.hh, BhabhaEnergyDistribution.hh
//   src/celeritas/em/interactor/EPlusGGInteractor.hh:99-170
//   src/celeritas/em/distribution/TsaiUrbanDistribution.hh
#pragma once

#include "Physics.hh"

namespace gbx
{
using RVec3 = Vec3<real_type>;

//! Outcome of one discrete interaction (src/celeritas/phys/Interaction.hh)
struct Interaction
{
    enum Action : int
    {
        scattered = 0,
        absorbed = 1,
        unchanged = 2,
        failed = 3,
    };
    real_type energy{0};
    RVec3 direction{0, 0, 0};
    Secondary* secondaries{nullptr};
    size_type num_secondaries{0};
    real_type energy_deposition{0};
    int action{scattered};

    static GBX_FORCEINLINE Interaction from_failure()
    {
        Interaction r;
        r.action = failed;
        return r;
    }
    static GBX_FORCEINLINE Interaction from_absorption()
    {
        Interaction r;
        r.energy = 0;
        r.action = absorbed;
        return r;
    }
};

//! Bump allocator over the secondary stack (src/corecel/data/StackAllocator.hh)
class SecondaryAllocator
{
  public:
    GBX_FORCEINLINE SecondaryAllocator(StateData const& s) : s_(s) {}

    GBX_FORCEINLINE Secondary* operator()(size_type count)
    {
        size_type* top = &s_.counters->secondary_stack_size;
#if defined(__CUDA_ARCH__)
        size_type start = atomicAdd(top, count);
#else
        size_type start = *top;
        *top += count;
#endif
        if (start + count > s_.secondary_capacity)
        {
            if (start <= s_.secondary_capacity)
            {
                *top = start;
            }
            return nullptr;
        }
        Secondary* result = s_.secondaries + start;
        for (size_type i = 0; i < count; ++i)
        {
            result[i].particle_id = invalid_id;
            result[i].energy = 0;
            result[i].direction = {0, 0, 0};
        }
        return result;
    }

  private:
    StateData const& s_;
};

//---------------------------------------------------------------------------//
//! Tsai-Urban polar angle of an outgoing lepton or photon
template<class G>
GBX_FORCEINLINE real_type sample_tsai_urban(real_type energy,
                                            real_type mass,
                                            G& rng)
{
    real_type const umax = 2 * (1 + energy / mass);
    real_type u;
    do
    {
        real_type uu = -libm::log(generate_canonical<real_type>(rng)
                                 * generate_canonical<real_type>(rng));
        u = uu
            * (sample_bernoulli<real_type>(real_type(0.25), rng)
                   ? real_type(1.6)
                   : real_type(1.6 / 3));
    } while (u > umax);
    return 1 - 2 * ipow<2>(u / umax);
}

//---------------------------------------------------------------------------//
// Klein-Nishina
//---------------------------------------------------------------------------//
template<class G>
GBX_FUNCTION Interaction interact_klein_nishina(ParamsData const& p,
                                                real_type inc_energy,
                                                RVec3 const& inc_dir,
                                                SecondaryAllocator& allocate,
                                                G& rng)
{
    Secondary* electron = allocate(1);
    if (electron == nullptr)
        return Interaction::from_failure();

    real_type const inv_electron_mass
        = real_type(1 / p.particles[p.electron_id].mass);
    real_type const k = inc_energy * inv_electron_mass;
    real_type const epsilon_0 = 1 / (1 + 2 * k);
    real_type const p_f1 = bernoulli_p(-libm::log(epsilon_0),
                                       real_type(0.5) * (1 - ipow<2>(epsilon_0)));
    ReciprocalDistribution<real_type> sample_f1(1, epsilon_0);
    UniformRealDistribution<real_type> sample_f2_sq(ipow<2>(epsilon_0), 1);

    real_type epsilon;
    real_type one_minus_costheta;
    real_type reject_prob;
    do
    {
        real_type epsilon_sq;
        if (sample_bernoulli<real_type>(p_f1, rng))
        {
            epsilon = sample_f1(rng);
            epsilon_sq = epsilon * epsilon;
        }
        else
        {
            epsilon_sq = sample_f2_sq(rng);
            epsilon = std::sqrt(epsilon_sq);
        }
        one_minus_costheta = (1 - epsilon) / (epsilon * k);
        real_type sintheta_sq = one_minus_costheta * (2 - one_minus_costheta);
        reject_prob = epsilon * sintheta_sq / (1 + epsilon_sq);
    } while (sample_bernoulli<real_type>(reject_prob, rng));

    Interaction result;
    result.energy = epsilon * inc_energy;
    result.secondaries = electron;
    result.num_secondaries = 1;
    result.direction
        = sample_exiting_direction<real_type>(1 - one_minus_costheta, inc_dir, rng);
    electron->energy = inc_energy - result.energy;
    if (electron->energy < real_type(1e-4))
    {
        result.energy_deposition = electron->energy;
        electron->particle_id = invalid_id;
        electron->energy = 0;
        return result;
    }
    electron->particle_id = p.electron_id;
    electron->direction = calc_exiting_direction<real_type>(
        inc_energy, inc_dir, result.energy, result.direction);
    return result;
}

//---------------------------------------------------------------------------//
// Livermore photoelectric
//---------------------------------------------------------------------------//
template<class G>
GBX_FUNCTION Interaction interact_livermore_pe(ParamsData const& p,
                                               size_type element,
                                               real_type inc_energy,
                                               RVec3 const& inc_dir,
                                               SecondaryAllocator& allocate,
                                               G& rng)
{
    Secondary* electron = allocate(1);
    if (electron == nullptr)
        return Interaction::from_failure();

    LivermoreElement const& el = p.livermore_elements[element];
    LivermoreShell const* shells = p.livermore_shells + el.shells;
    real_type const inv_energy = 1 / inc_energy;
    real_type const inv_electron_mass
        = real_type(1 / p.particles[p.electron_id].mass);

    // Sample the subshell
    size_type shell_id = 0;
    real_type const cutoff = generate_canonical<real_type>(rng)
                             * livermore_pe_micro_xs(p, element, inc_energy);
    if (inc_energy < el.thresh_lo)
    {
        real_type xs = 0;
        real_type const inv_cube_energy = ipow<3>(inv_energy);
        for (; shell_id < el.num_shells; ++shell_id)
        {
            LivermoreShell const& shell = shells[shell_id];
            if (inc_energy < shell.binding_energy)
                continue;
            xs += inv_cube_energy * calc_generic(p, shell.xs, inc_energy);
            if (xs > cutoff)
                break;
        }
        if (shell_id == el.num_shells)
        {
            Interaction result = Interaction::from_absorption();
            result.energy_deposition = inc_energy;
            return result;
        }
    }
    else
    {
        int const pidx = inc_energy < el.thresh_hi ? 0 : 1;
        size_type const shell_end = el.num_shells - 1;
        for (; shell_id < shell_end; ++shell_id)
        {
            real_type c[6];
            for (int i = 0; i < 6; ++i)
                c[i] = shells[shell_id].param[pidx][i];
            real_type xs = inv_energy * poly_eval<5>(c, inv_energy);
            if (xs > cutoff)
                break;
        }
    }
    real_type const binding_energy = shells[shell_id].binding_energy;

    // Photoelectron direction (Sauter-Gavrila)
    RVec3 edir;
    if (inc_energy > real_type(100.))
    {
        edir = inc_dir;
    }
    else
    {
        real_type energy_per_mecsq = max_of(real_type(1.e-6), inc_energy)
                                     * inv_electron_mass;
        real_type gamma = energy_per_mecsq + 1;
        real_type beta = std::sqrt(energy_per_mecsq * (gamma + 1)) / gamma;
        real_type a = (1 - beta) / beta;
        constexpr real_type half = 0.5;
        real_type b = half * beta * gamma * energy_per_mecsq * (gamma - 2);
        real_type g_max = 2 * (1 / a + b);
        real_type g;
        real_type nu;
        do
        {
            real_type u = generate_canonical<real_type>(rng);
            nu = 2 * a * (2 * u + (a + 2) * std::sqrt(u))
                 / (ipow<2>(a + 2) - 4 * u);
            g = (2 - nu) * (1 / (a + nu) + b);
        } while (g < g_max * generate_canonical<real_type>(rng));
        edir = sample_exiting_direction<real_type>(1 - nu, inc_dir, rng);
    }
    electron->particle_id = p.electron_id;
    electron->energy = inc_energy - binding_energy;
    electron->direction = edir;

    Interaction result = Interaction::from_absorption();
    result.energy_deposition = binding_energy;
    result.secondaries = electron;
    result.num_secondaries = 1;
    return result;
}

//---------------------------------------------------------------------------//
// Bethe-Heitler pair production (no LPM suppression below 100 GeV)
//---------------------------------------------------------------------------//
GBX_FORCEINLINE real_type bh_screening_f1(real_type delta)
{
    using R = real_type;
    return delta > R(1.4) ? R(42.038) - R(8.29) * libm::log(delta + R(0.958))
                          : R(42.184) - delta * (R(7.444) - R(1.623) * delta);
}
GBX_FORCEINLINE real_type bh_screening_f2(real_type delta)
{
    using R = real_type;
    return delta > R(1.4) ? R(42.038) - R(8.29) * libm::log(delta + R(0.958))
                          : R(41.326) - delta * (R(5.848) - R(0.902) * delta);
}

template<class G>
GBX_FUNCTION Interaction interact_bethe_heitler(ParamsData const& p,
                                                ElementRecord const& element,
                                                real_type inc_energy,
                                                RVec3 const& inc_dir,
                                                SecondaryAllocator& allocate,
                                                G& rng)
{
    Secondary* secondaries = allocate(2);
    if (secondaries == nullptr)
        return Interaction::from_failure();

    real_type const electron_mass = p.particles[p.electron_id].mass;
    real_type const epsilon0 = electron_mass / inc_energy;
    real_type const cbrt_z = element.cbrt_z;
    constexpr real_type half = 0.5;
    real_type epsilon;
    if (inc_energy < real_type(2))
    {
        epsilon = UniformRealDistribution<real_type>(epsilon0, half)(rng);
    }
    else
    {
        real_type const delta_min = 4 * 136 / cbrt_z * epsilon0;
        real_type f_z = real_type(8) / real_type(3) * real_type(element.log_z);
        if (inc_energy > real_type(50))
        {
            f_z += 8 * real_type(element.coulomb_correction);
        }
        real_type const delta_max
            = libm::exp((real_type(42.038) - f_z) / real_type(8.29))
              - real_type(0.958);
        real_type const epsilon1
            = half - half * std::sqrt(1 - delta_min / delta_max);
        real_type const epsilon_min = max_of(epsilon0, epsilon1);
        real_type const f10 = bh_screening_f1(delta_min) - f_z;
        real_type const f20 = bh_screening_f2(delta_min) - f_z;
        real_type const p_f1g1
            = bernoulli_p(ipow<2>(half - epsilon_min) * f10, real_type(1.5) * f20);
        auto impact_parameter = [&](real_type eps) {
            return 136 / cbrt_z * epsilon0 / (eps * (1 - eps));
        };
        real_type g;
        do
        {
            if (sample_bernoulli<real_type>(p_f1g1, rng))
            {
                epsilon = half
                          - (half - epsilon_min)
                                * libm::cbrt(generate_canonical<real_type>(rng));
                real_type delta = impact_parameter(epsilon);
                g = (bh_screening_f1(delta) - f_z) / f10;
            }
            else
            {
                epsilon = epsilon_min
                          + (half - epsilon_min) * generate_canonical<real_type>(rng);
                real_type delta = impact_parameter(epsilon);
                g = (bh_screening_f2(delta) - f_z) / f20;
            }
        } while (g < generate_canonical<real_type>(rng));
    }

    Interaction result = Interaction::from_absorption();
    result.secondaries = secondaries;
    result.num_secondaries = 2;
    secondaries[0].particle_id = p.electron_id;
    secondaries[1].particle_id = p.positron_id;
    secondaries[0].energy = (1 - epsilon) * inc_energy - electron_mass;
    secondaries[1].energy = epsilon * inc_energy - electron_mass;
    if (sample_bernoulli<real_type>(half, rng))
    {
        real_type tmp = secondaries[0].energy;
        secondaries[0].energy = secondaries[1].energy;
        secondaries[1].energy = tmp;
    }
    real_type phi = UniformRealDistribution<real_type>(0, 2 * constants::pi)(rng);
    real_type cost = sample_tsai_urban(secondaries[0].energy, electron_mass, rng);
    secondaries[0].direction = rotate(from_spherical(cost, phi), inc_dir);
    cost = sample_tsai_urban(secondaries[1].energy, electron_mass, rng);
    secondaries[1].direction = rotate(
        from_spherical(cost, phi + real_type(constants::pi)), inc_dir);
    return result;
}

//---------------------------------------------------------------------------//
//! Energy [MeV] above which the combined bremsstrahlung model samples with
//! the relativistic model (seltzer_berger_upper_limit, 1 GeV,
//! src/celeritas/em/interactor/detail/PhysicsConstants.hh)
constexpr double seltzer_berger_upper_limit = 1000;

// Seltzer-Berger bremsstrahlung
//---------------------------------------------------------------------------//
//! Bilinear lookup of the scaled DCS table at (log E, reduced energy)
struct SBXsCalc
{
    ParamsData const& p;
    SBElementTable const& t;
    size_type x_index;
    real_type x_fraction;

    GBX_FORCEINLINE real_type at(size_type ix, size_type iy) const
    {
        return p.reals[t.values + ix * t.ny + iy];
    }

    GBX_FORCEINLINE real_type operator()(real_type y) const
    {
        real_type const* ygrid = p.reals + t.y;
        size_type iy = find_nonuniform(ygrid, t.ny, y);
        real_type const lower = ygrid[iy];
        real_type const upper = ygrid[iy + 1];
        real_type const yf = (y - lower) / (upper - lower);
        real_type const xf = x_fraction;
        return (1 - xf) * ((1 - yf) * at(x_index, iy) + (yf)*at(x_index, iy + 1))
               + (xf) * ((1 - yf) * at(x_index + 1, iy) + (yf)*at(x_index + 1, iy + 1));
    }
};

template<class G>
GBX_FUNCTION Interaction interact_seltzer_berger(ParamsData const& p,
                                                 size_type element_id,
                                                 MaterialRecord const& mat,
                                                 bool is_electron,
                                                 real_type inc_mass,
                                                 real_type inc_energy,
                                                 RVec3 const& inc_dir,
                                                 real_type gamma_cutoff,
                                                 SecondaryAllocator& allocate,
                                                 G& rng)
{
    Secondary* photon = allocate(1);
    if (photon == nullptr)
        return Interaction::from_failure();

    real_type const inc_momentum
        = std::sqrt(momentum_sq(inc_mass, inc_energy));
    // Density (dielectric suppression) correction
    constexpr real_type migdal = 4 * constants::pi * constants::r_electron
                                 * ipow<2>(constants::lambdabar_electron);
    real_type const density_factor = real_type(mat.electron_density) * migdal;
    real_type const total_energy = inc_energy + inc_mass;
    real_type const dens_corr = density_factor * ipow<2>(total_energy);

    // Table position in log energy
    SBElementTable const& t = p.sb_tables[element_id];
    real_type const* xgrid = p.reals + t.x;
    real_type const loge = libm::log(inc_energy);
    size_type ix = find_nonuniform(xgrid, t.nx, loge);
    real_type const xf = (loge - real_type(xgrid[ix]))
                         / (real_type(xgrid[ix + 1]) - real_type(xgrid[ix]));
    SBXsCalc calc_xs{p, t, ix, xf};
    real_type max_xs;
    {
        auto get_value = [&](size_type jx) -> real_type {
            size_type iy = p.ints[t.argmax + jx];
            return calc_xs.at(jx, iy);
        };
        max_xs = (1 - xf) * get_value(ix) + xf * get_value(ix + 1);
    }
    real_type const inv_inc_energy = 1 / inc_energy;
    ReciprocalDistribution<real_type> sample_exit_esq(
        ipow<2>(gamma_cutoff) + dens_corr, ipow<2>(inc_energy) + dens_corr);

    // Positron correction (exp of alpha Z times the change in 1/beta)
    real_type const alpha_z = 2 * real_type(constants::pi)
                              * real_type(constants::alpha_fine_structure)
                              * real_type(p.elements[element_id].z);
    auto calc_invbeta = [&](real_type gamma_energy) {
        real_type energy = inc_energy - gamma_energy;
        return (energy + inc_mass) / std::sqrt(energy * (energy + 2 * inc_mass));
    };
    real_type const cutoff_invbeta = is_electron ? 0 : calc_invbeta(gamma_cutoff);

    real_type gamma_energy;
    real_type xs;
    do
    {
        real_type esq = sample_exit_esq(rng) - dens_corr;
        gamma_energy = std::sqrt(esq);
        xs = calc_xs(gamma_energy * inv_inc_energy);
        if (is_electron)
        {
            xs = xs * real_type(1);
        }
        else
        {
            real_type delta = cutoff_invbeta - calc_invbeta(gamma_energy);
            xs = xs * libm::exp(alpha_z * min_of(delta, real_type{0}));
        }
    } while (reject_sample<real_type>(xs, max_xs, rng));

    real_type const costheta = sample_tsai_urban(inc_energy, inc_mass, rng);

    photon->direction = sample_exiting_direction<real_type>(costheta, inc_dir, rng);
    photon->particle_id = p.gamma_id;
    photon->energy = gamma_energy;
    Interaction result;
    result.energy = inc_energy - gamma_energy;
    result.direction = calc_exiting_direction<real_type>(
        inc_momentum, inc_dir, gamma_energy, photon->direction);
    result.secondaries = photon;
    result.num_secondaries = 1;
    return result;
}

//---------------------------------------------------------------------------//
// Relativistic bremsstrahlung with LPM suppression
// (src/celeritas/em/interactor/RelativisticBremInteractor.hh,
//  interactor/detail/RBEnergySampler.hh, xs/RBDiffXsCalculator.hh,
//  xs/LPMCalculator.hh)
//---------------------------------------------------------------------------//
namespace detail
{
// CGS unit system constants in the reference's definition order
constexpr double unit_kilogram = 1000 * constants::gram;
constexpr double unit_newton
    = unit_kilogram * constants::meter / (constants::second * constants::second);
constexpr double unit_joule = unit_newton * constants::meter;
constexpr double unit_coulomb = unit_kilogram / (constants::tesla * constants::second);
constexpr double unit_volt = unit_joule / unit_coulomb;
constexpr double e_electron = 1.602176634e-19 * unit_coulomb;
constexpr double mev_value = double(1e6) * e_electron * unit_volt;
constexpr double h_planck = 6.62607015e-34 * unit_joule * constants::second;
constexpr double electron_mass_g = 9.1093837015e-28 * constants::gram;

//! LPM constant [MeV/cm]: alpha (m c^2)^2 / (2 h c)
constexpr double lpm_constant()
{
    constexpr double electron_mass_csq
        = electron_mass_g * ipow<2>(constants::c_light);
    return constants::alpha_fine_structure * ipow<2>(electron_mass_csq)
           / (2 * h_planck * constants::c_light) / mev_value;
}

constexpr double migdal_constant()
{
    return 4 * constants::pi * constants::r_electron
           * ipow<2>(constants::lambdabar_electron);
}

struct LPMFunctions
{
    real_type xi;
    real_type g;
    real_type phi;
};

//! LPM suppression functions (Stanev / Klein parameterizations)
GBX_FUNCTION LPMFunctions calc_lpm(MaterialRecord const& mat,
                                   ElementRecord const& el,
                                   real_type gamma_energy,
                                   real_type epsilon)
{
    constexpr real_type sqrt_two = 1.41421356237309504880;
    real_type const lpm_energy = real_type(mat.rad_length) * real_type(lpm_constant());
    real_type const s_prime = std::sqrt(
        lpm_energy / (8 * epsilon * gamma_energy * std::fabs(epsilon - 1)));
    real_type const s1 = ipow<2>(real_type(el.cbrt_z) / real_type(184.15));
    real_type xi = 2;
    if (s_prime > 1)
    {
        xi = 1;
    }
    else if (s_prime > sqrt_two * s1)
    {
        real_type const log_s1 = libm::log(sqrt_two * s1);
        real_type const h = libm::log(s_prime) / log_s1;
        xi = 1 + h - real_type(0.08) * (1 - h) * h * (2 - h) / log_s1;
    }
    real_type s = s_prime / std::sqrt(xi);
    // Dielectric suppression is always on for relativistic bremsstrahlung
    {
        real_type const k_p_sq = real_type(mat.electron_density)
                                 * real_type(migdal_constant())
                                 * ipow<2>(epsilon * gamma_energy);
        s *= (1 + k_p_sq / ipow<2>(gamma_energy));
        xi = 2;
        if (s > 1)
        {
            xi = 1;
        }
        else if (s > s1)
        {
            xi = 1 + libm::log(s) / libm::log(s1);
        }
    }
    real_type phi;
    if (s < real_type(0.01))
    {
        real_type const c[2] = {6, real_type(-6 * constants::pi)};
        phi = s * poly_eval<1>(c, s);
    }
    else if (s < real_type(1.55))
    {
        real_type const ca[3] = {real_type(0.623), real_type(0.796), real_type(0.658)};
        real_type a = poly_eval<2>(ca, s);
        real_type const cb[3]
            = {real_type(-6), real_type(-6 * (3 - constants::pi)), 1 / a};
        real_type b = poly_eval<2>(cb, s);
        phi = 1 - libm::exp(s * b);
    }
    else
    {
        phi = 1 - real_type(0.01190476) / ipow<4>(s);
    }
    if (xi * phi > 1 || s > real_type(0.57))
    {
        xi = 1 / phi;
    }
    real_type g;
    if (s < real_type(0.01))
    {
        real_type const c[2] = {-2 * phi, 12};
        g = poly_eval<1>(c, s);
    }
    else if (s < real_type(0.415827))
    {
        real_type const ca[5] = {real_type(1),
                                 real_type(3.936),
                                 real_type(4.97),
                                 real_type(-0.05),
                                 real_type(7.5)};
        real_type a = poly_eval<4>(ca, s);
        real_type const cb[2] = {real_type(-4), -8 / a};
        real_type b = poly_eval<1>(cb, s);
        real_type psi = 1 - libm::exp(s * b);
        g = 3 * psi - 2 * phi;
    }
    else if (s < real_type(1.9156))
    {
        real_type const c[5] = {real_type(-0.160723),
                                real_type(3.755030),
                                real_type(-1.798138),
                                real_type(0.672827),
                                real_type(-0.120772)};
        g = libm::tanh(poly_eval<4>(c, s));
    }
    else
    {
        g = 1 - real_type(0.0230655) / ipow<4>(s);
    }
    return {xi, g, phi};
}
}  // namespace detail

template<class G>
GBX_FUNCTION Interaction interact_relativistic_brems(ParamsData const& p,
                                                     size_type element_id,
                                                     MaterialRecord const& mat,
                                                     real_type inc_mass,
                                                     real_type inc_energy,
                                                     RVec3 const& inc_dir,
                                                     real_type gamma_cutoff,
                                                     SecondaryAllocator& allocate,
                                                     G& rng)
{
    Secondary* photon = allocate(1);
    if (photon == nullptr)
        return Interaction::from_failure();
    using R = real_type;
    RelBremElementRecord const& ed = p.rb_elements[element_id];
    ElementRecord const& el = p.elements[element_id];
    real_type const inc_momentum = std::sqrt(momentum_sq(inc_mass, inc_energy));
    real_type const total_energy = inc_energy + inc_mass;
    real_type const density_factor
        = R(mat.electron_density) * R(detail::migdal_constant());
    real_type const density_corr = density_factor * ipow<2>(total_energy);
    real_type const lpm_energy = R(mat.rad_length) * R(detail::lpm_constant());
    real_type const lpm_threshold = lpm_energy * std::sqrt(density_factor);
    bool const enable_lpm = p.enable_lpm && (total_energy > lpm_threshold);

    auto dxsec_per_atom = [&](real_type gamma_energy) -> real_type {
        real_type dxsec{0};
        real_type y = gamma_energy / total_energy;
        real_type onemy = 1 - y;
        real_type term0 = onemy + R(0.75) * ipow<2>(y);
        if (el.z < 5)
        {
            dxsec = term0 * R(ed.factor1) + onemy * R(ed.factor2);
        }
        else
        {
            real_type invz = 1 / static_cast<real_type>(el.z);
            real_type term1 = y / (total_energy - gamma_energy);
            real_type gam = term1 * R(ed.gamma_factor);
            real_type eps = term1 * R(ed.epsilon_factor);
            real_type gam2 = ipow<2>(gam);
            real_type eps2 = ipow<2>(eps);
            real_type phi1 = R(16.863) - 2 * libm::log(1 + R(0.311877) * gam2)
                             + R(2.4) * libm::exp(R(-0.9) * gam)
                             + R(1.6) * libm::exp(R(-1.5) * gam);
            real_type phi2 = 2 / (3 + R(19.5) * gam + 18 * gam2);
            real_type psi1 = R(24.34) - 2 * libm::log(1 + R(13.111641) * eps2)
                             + R(2.8) * libm::exp(R(-8) * eps)
                             + R(1.2) * libm::exp(R(-29.2) * eps);
            real_type psi2 = 2 / (3 + 120 * eps + 1200 * eps2);
            dxsec = term0
                        * ((R(0.25) * phi1 - R(ed.fz))
                           + (R(0.25) * psi1 - 2 * R(el.log_z) / 3) * invz)
                    + R(0.125) * onemy * (phi2 + psi2 * invz);
        }
        return max_of(dxsec, R(0));
    };
    auto dxsec_per_atom_lpm = [&](real_type gamma_energy) -> real_type {
        real_type epsilon = total_energy / gamma_energy;
        detail::LPMFunctions lpm = detail::calc_lpm(mat, el, gamma_energy, epsilon);
        real_type y = gamma_energy / total_energy;
        real_type onemy = 1 - y;
        real_type y2 = R(0.25) * ipow<2>(y);
        real_type term = lpm.xi * (y2 * lpm.g + (onemy + 2 * y2) * lpm.phi);
        real_type dxsec = term * R(ed.factor1) + onemy * R(ed.factor2);
        return max_of(dxsec, R(0));
    };

    // RBEnergySampler
    real_type const tmin_sq = ipow<2>(min_of(gamma_cutoff, inc_energy));
    real_type const tmax_sq = ipow<2>(min_of(R(1e8), inc_energy));
    ReciprocalDistribution<real_type> sample_exit_esq(tmin_sq + density_corr,
                                                      tmax_sq + density_corr);
    real_type const max_value = R(ed.factor1) + R(ed.factor2);
    real_type gamma_energy{0};
    real_type dsigma{0};
    do
    {
        gamma_energy = std::sqrt(sample_exit_esq(rng) - density_corr);
        dsigma = enable_lpm ? dxsec_per_atom_lpm(gamma_energy)
                            : dxsec_per_atom(gamma_energy);
    } while (reject_sample<real_type>(dsigma, max_value, rng));

    real_type const costheta = sample_tsai_urban(inc_energy, inc_mass, rng);

    photon->direction = sample_exiting_direction<real_type>(costheta, inc_dir, rng);
    photon->particle_id = p.gamma_id;
    photon->energy = gamma_energy;
    Interaction result;
    result.energy = inc_energy - gamma_energy;
    result.direction = calc_exiting_direction<real_type>(
        inc_momentum, inc_dir, gamma_energy, photon->direction);
    result.secondaries = photon;
    result.num_secondaries = 1;
    return result;
}

//---------------------------------------------------------------------------//
// Moller-Bhabha ionization
//---------------------------------------------------------------------------//
template<class G>
GBX_FUNCTION Interaction interact_moller_bhabha(ParamsData const& p,
                                                bool is_electron,
                                                real_type inc_energy,
                                                RVec3 const& inc_dir,
                                                real_type electron_cutoff,
                                                SecondaryAllocator& allocate,
                                                G& rng)
{
    Secondary* electron = allocate(1);
    if (electron == nullptr)
        return Interaction::from_failure();

    real_type const electron_mass = p.particles[p.electron_id].mass;
    real_type const inc_momentum
        = std::sqrt(momentum_sq(electron_mass, inc_energy));
    real_type const min_energy_fraction = electron_cutoff / inc_energy;
    real_type const gamma = 1 + inc_energy / electron_mass;
    real_type epsilon;
    if (is_electron)
    {
        auto calc_g_fraction = [gamma](real_type eps) {
            real_type const two_gamma_term = (2 * gamma - 1) / ipow<2>(gamma);
            real_type const complement_frac = 1 - eps;
            return 1 - two_gamma_term * eps
                   + ipow<2>(eps)
                         * (1 - two_gamma_term
                            + (1 - two_gamma_term * complement_frac)
                                  / ipow<2>(complement_frac));
        };
        constexpr real_type max_energy_fraction = 0.5;
        real_type const g_denominator = calc_g_fraction(max_energy_fraction);
        UniformRealDistribution<real_type> sample_inverse_epsilon(
            1 / max_energy_fraction, 1 / min_energy_fraction);
        do
        {
            epsilon = 1 / sample_inverse_epsilon(rng);
        } while (reject_sample<real_type>(calc_g_fraction(epsilon), g_denominator, rng));
    }
    else
    {
        auto calc_g_fraction = [gamma](real_type eps_min, real_type eps_max) {
            real_type const y = 1 / (1 + gamma);
            real_type const y_sq = ipow<2>(y);
            real_type const one_minus_2y = 1 - 2 * y;
            real_type const b1 = 2 - y_sq;
            real_type const b2 = one_minus_2y * (3 + y_sq);
            real_type const b4 = ipow<3>(one_minus_2y);
            real_type const b3 = ipow<2>(one_minus_2y) + b4;
            real_type const beta_sq = 1 - (1 / ipow<2>(gamma));
            return 1
                   + (ipow<4>(eps_max) * b4 - ipow<3>(eps_min) * b3
                      + ipow<2>(eps_max) * b2 - eps_min * b1)
                         * beta_sq;
        };
        constexpr real_type max_energy_fraction = 1;
        real_type const g_denominator
            = calc_g_fraction(min_energy_fraction, max_energy_fraction);
        UniformRealDistribution<real_type> sample_inverse_epsilon(
            1 / max_energy_fraction, 1 / min_energy_fraction);
        do
        {
            epsilon = 1 / sample_inverse_epsilon(rng);
        } while (reject_sample<real_type>(
            calc_g_fraction(epsilon, epsilon), g_denominator, rng));
    }
    real_type const secondary_energy = inc_energy * epsilon;

    // Final state (src/celeritas/em/interactor/detail/IoniFinalStateHelper.hh)
    real_type const momentum
        = std::sqrt(secondary_energy * (secondary_energy + 2 * electron_mass));
    real_type const costheta = secondary_energy
                               * (inc_energy + electron_mass + electron_mass)
                               / (momentum * inc_momentum);
    electron->energy = secondary_energy;
    electron->direction = sample_exiting_direction<real_type>(costheta, inc_dir, rng);
    electron->particle_id = p.electron_id;
    Interaction result;
    result.energy = inc_energy - secondary_energy;
    result.direction = calc_exiting_direction<real_type>(
        inc_momentum, inc_dir, momentum, electron->direction);
    result.secondaries = electron;
    result.num_secondaries = 1;
    return result;
}

//---------------------------------------------------------------------------//
// Positron annihilation to two photons
//---------------------------------------------------------------------------//
template<class G>
GBX_FUNCTION Interaction interact_eplusgg(ParamsData const& p,
                                          real_type inc_energy,
                                          RVec3 const& inc_dir,
                                          SecondaryAllocator& allocate,
                                          G& rng)
{
    Secondary* secondaries = allocate(2);
    if (secondaries == nullptr)
        return Interaction::from_failure();

    real_type const electron_mass = p.particles[p.electron_id].mass;
    Interaction result = Interaction::from_absorption();
    result.secondaries = secondaries;
    result.num_secondaries = 2;
    secondaries[0].particle_id = secondaries[1].particle_id = p.gamma_id;
    if (inc_energy == 0)
    {
        secondaries[0].energy = secondaries[1].energy = electron_mass;
        RVec3 d = sample_isotropic<real_type>(rng);
        secondaries[0].direction = d;
        secondaries[1].direction = {-d.x, -d.y, -d.z};
    }
    else
    {
        constexpr real_type half = 0.5;
        real_type const tau = inc_energy / electron_mass;
        real_type const tau2 = tau + 2;
        real_type const sqgrate = std::sqrt(tau / tau2) * half;
        ReciprocalDistribution<real_type> sample_eps(half - sqgrate,
                                                     half + sqgrate);
        real_type epsil;
        do
        {
            epsil = sample_eps(rng);
        } while (sample_bernoulli<real_type>(
            epsil - (2 * (tau + 1) * epsil - 1) / (epsil * ipow<2>(tau2)), rng));
        real_type const cost = (epsil * tau2 - 1) / (epsil * std::sqrt(tau * tau2));
        real_type const total_energy = inc_energy + 2 * electron_mass;
        real_type const gamma_energy = epsil * total_energy;
        real_type const eplus_moment = std::sqrt(inc_energy * total_energy);
        secondaries[0].energy = gamma_energy;
        secondaries[0].direction
            = sample_exiting_direction<real_type>(cost, inc_dir, rng);
        secondaries[1].energy = total_energy - gamma_energy;
        secondaries[1].direction = calc_exiting_direction<real_type>(
            eplus_moment, inc_dir, inc_energy, inc_dir);
    }
    return result;
}

}  // namespace gbx
