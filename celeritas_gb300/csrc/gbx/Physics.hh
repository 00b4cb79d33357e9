// Cross-section tables, step limits, continuous energy loss and discrete
// process selection.
//
// Table interpolation follows src/celeritas/grid/XsCalculator.hh:107-153,
// RangeCalculator.hh:80-108, InverseRangeCalculator.hh and
// GenericCalculator.hh; the grid energies exp(log_front + i * log_delta) are
// precomputed on the host (same expression, same libm) so the device does
// one log per lookup instead of one log and two exps.
// Step limits follow src/celeritas/phys/PhysicsStepUtils.hh:37-120 and
// PhysicsTrackView.hh:399-470, energy loss PhysicsStepUtils.hh:177-233 with
// the Urban fluctuation model of
// src/celeritas/em/distribution/EnergyLossUrbanDistribution.hh, discrete
// selection PhysicsStepUtils.hh:253-308.
#pragma once

#include "Data.hh"

namespace gbx
{
//---------------------------------------------------------------------------//
// Interpolation helpers
//---------------------------------------------------------------------------//
//! Linear interpolation y0 + (x - x0) * slope, as fma(slope, -x0 + x, y0)
template<class T>
GBX_FORCEINLINE T interp_linear(T x0, T y0, T x1, T y1, T x)
{
    T slope = (-y0 + y1) / (-x0 + x1);
    return gbx_fma(slope, (-x0 + x), y0);
}

//! Index of the largest grid value <= v (lower_bound, then step back unless
//! exact); clamped so that index + 1 is valid.
template<class T>
GBX_FORCEINLINE size_type find_nonuniform(T const* grid, size_type size, T v)
{
    size_type lo = 0, count = size;
    while (count > 0)
    {
        size_type step = count / 2;
        size_type it = lo + step;
        if (grid[it] < v)
        {
            lo = it + 1;
            count -= step + 1;
        }
        else
        {
            count = step;
        }
    }
    if (lo >= size || v != grid[lo])
    {
        lo = (lo == 0) ? 0 : lo - 1;
    }
    return min_of(lo, size - 2);
}

//! Macroscopic cross section (or dE/dx) from a log-uniform grid, given
//! log(energy)
GBX_FORCEINLINE real_type calc_grid_xs(ParamsData const& p,
                                       XsGrid const& g,
                                       real_type energy,
                                       real_type loge)
{
    real_type const* values = p.reals + g.value;
    real_type const* energies = p.reals + g.energy;
    auto extrapolated = [&](size_type idx) {
        real_type result = values[idx];
        if (idx >= g.prime_index)
            result /= energy;
        return result;
    };
    if (loge <= g.log_front)
        return extrapolated(0);
    if (loge >= g.log_back)
        return extrapolated(g.size - 1);
    size_type lower = static_cast<size_type>((loge - g.log_front) / g.log_delta);
    lower = min_of(lower, g.size - 2);
    real_type upper_energy = energies[lower + 1];
    real_type upper_xs = values[lower + 1];
    if (lower + 1 == g.prime_index)
        upper_xs /= upper_energy;
    real_type result = interp_linear<real_type>(
        energies[lower], values[lower], upper_energy, upper_xs, energy);
    if (lower >= g.prime_index)
        result /= energy;
    return result;
}

//! Macroscopic cross section (or dE/dx) from a log-uniform grid
GBX_FORCEINLINE real_type calc_grid_xs(ParamsData const& p,
                                       XsGrid const& g,
                                       real_type energy)
{
    return calc_grid_xs(p, g, energy, libm::log(energy));
}

//! Range from a log-uniform grid, with sqrt(E) scaling below the grid,
//! given log(energy)
GBX_FORCEINLINE real_type calc_range(ParamsData const& p,
                                     XsGrid const& g,
                                     real_type energy,
                                     real_type loge)
{
    real_type const* values = p.reals + g.value;
    real_type const* energies = p.reals + g.energy;
    if (loge <= g.log_front)
    {
        real_type result = values[0];
        result *= libm::exp(real_type(.5) * (loge - g.log_front));
        return result;
    }
    if (loge >= g.log_back)
        return values[g.size - 1];
    size_type idx = static_cast<size_type>((loge - g.log_front) / g.log_delta);
    idx = min_of(idx, g.size - 2);
    return interp_linear<real_type>(
        energies[idx], values[idx], energies[idx + 1], values[idx + 1], energy);
}

//! Range from a log-uniform grid, with sqrt(E) scaling below the grid
GBX_FORCEINLINE real_type calc_range(ParamsData const& p,
                                     XsGrid const& g,
                                     real_type energy)
{
    return calc_range(p, g, energy, libm::log(energy));
}

//! Energy from range (inverse of the range table)
GBX_FORCEINLINE real_type calc_inverse_range(ParamsData const& p,
                                             XsGrid const& g,
                                             real_type range)
{
    real_type const* values = p.reals + g.value;
    real_type const* energies = p.reals + g.energy;
    if (range < values[0])
    {
        return energies[0] * ipow<2>(range / values[0]);
    }
    if (range >= values[g.size - 1])
    {
        // exp of the stored upper bound, kept after the grid energies
        return energies[g.size];
    }
    size_type idx = find_nonuniform(values, g.size, range);
    return interp_linear<real_type>(
        values[idx], energies[idx], values[idx + 1], energies[idx + 1], range);
}

//! Linear interpolation on a nonuniform grid, clamped at the ends
GBX_FORCEINLINE real_type calc_generic(ParamsData const& p,
                                       GenericGrid const& g,
                                       real_type x)
{
    real_type const* xs = p.reals + g.x;
    real_type const* ys = p.reals + g.y;
    if (x <= xs[0])
        return ys[0];
    if (x >= xs[g.size - 1])
        return ys[g.size - 1];
    size_type idx = find_nonuniform(xs, g.size, x);
    return interp_linear<real_type>(xs[idx], ys[idx], xs[idx + 1], ys[idx + 1], x);
}

//---------------------------------------------------------------------------//
// On-the-fly cross sections
//---------------------------------------------------------------------------//
//! Livermore photoelectric micro cross section [b]
//! (src/celeritas/em/xs/LivermorePEMicroXsCalculator.hh:67)
GBX_FORCEINLINE real_type livermore_pe_micro_xs(ParamsData const& p,
                                                size_type element,
                                                real_type inc_energy)
{
    LivermoreElement const& el = p.livermore_elements[element];
    LivermoreShell const* shells = p.livermore_shells + el.shells;
    real_type energy = max_of(inc_energy,
                              real_type(shells[el.num_shells - 1].binding_energy));
    real_type inv_energy = real_type(1.) / energy;
    real_type result = 0.;
    if (energy >= el.thresh_lo)
    {
        real_type const* param
            = shells[el.num_shells - 1].param[energy < el.thresh_hi ? 0 : 1];
        real_type c[6];
        for (int i = 0; i < 6; ++i)
            c[i] = param[i];
        result = inv_energy * poly_eval<5>(c, inv_energy);
    }
    else if (energy >= shells[0].binding_energy)
    {
        result = ipow<3>(inv_energy) * calc_generic(p, el.xs_hi, energy);
    }
    else
    {
        result = ipow<3>(inv_energy) * calc_generic(p, el.xs_lo, energy);
    }
    return result;
}

//! Macroscopic cross section from micro cross sections in barns
//! (src/celeritas/phys/MacroXsCalculator.hh)
GBX_FORCEINLINE real_type livermore_pe_macro_xs(ParamsData const& p,
                                                MaterialRecord const& mat,
                                                real_type energy)
{
    real_type result = 0.;
    for (size_type i = 0; i < mat.num_elements; ++i)
    {
        real_type micro = livermore_pe_micro_xs(p, mat.element[i], energy);
        result += micro * real_type(mat.fraction[i]);
    }
    result = result * real_type(constants::barn) * real_type(mat.number_density);
    return result;
}

//! Positron annihilation (Heitler) macro cross section
//! (src/celeritas/em/xs/EPlusGGMacroXsCalculator.hh)
GBX_FORCEINLINE real_type eplusgg_macro_xs(ParamsData const& p,
                                           MaterialRecord const& mat,
                                           real_type energy)
{
    real_type const electron_mass = p.particles[p.electron_id].mass;
    real_type const gamma = max_of(energy, real_type(1e-6)) / electron_mass;
    real_type const sqrt_gg2 = std::sqrt(gamma * (gamma + 2));
    real_type const quad[3] = {1, 4, 1};
    real_type result
        = real_type(constants::pi) * ipow<2>(real_type(constants::r_electron))
          * real_type(mat.electron_density)
          * (poly_eval<2>(quad, gamma + 1) * libm::log(gamma + 1 + sqrt_gg2)
             - (gamma + 4) * sqrt_gg2)
          / (gamma * ipow<2>(gamma + 2));
    return result;
}

//---------------------------------------------------------------------------//
// Per-track physics helper
//---------------------------------------------------------------------------//
class PhysicsTrack
{
  public:
    GBX_FORCEINLINE PhysicsTrack(ParamsData const& p,
                                 size_type particle,
                                 size_type material)
        : p_(p)
        , group_(p.process_groups[particle])
        , particle_(particle)
        , material_(material)
    {
    }

    //! Physics of the track in 'slot', whose log(energy) the FP64 build
    //! keeps per slot between the step's actions (a correctly rounded FP64
    //! logarithm costs tens of FP64 instructions, of which GB300 issues two
    //! per SM and clock; the mixed build's FP32 logarithm costs less than
    //! the memory traffic would)
    GBX_FORCEINLINE PhysicsTrack(ParamsData const& p,
                                 size_type particle,
                                 size_type material,
                                 StateData const& s,
                                 size_type slot)
        : PhysicsTrack(p, particle, material)
    {
        if constexpr (sizeof(real_type) == sizeof(double))
        {
            cache_key_ = s.log_energy_key + slot;
            cache_val_ = s.log_energy_value + slot;
            slot_energy_ = s.energy[slot];
        }
    }

    GBX_FORCEINLINE size_type num_processes() const
    {
        return group_.num_processes;
    }

    //! log(energy), remembered for the last two energies: the table lookups
    //! of one step take the logarithm of the same few energies many times
    //! (every process at E and at E * min_eprime_over_e, the range and the
    //! stopping power at E), and the function returns the same double for
    //! the same argument, so a remembered value changes no result. With a
    //! slot cache, the log of the slot's energy is also kept across the
    //! step's actions, keyed by the exact energy.
    GBX_FORCEINLINE real_type log_energy(real_type energy) const
    {
        if (energy == memo_e_[0])
            return memo_log_[0];
        if (energy == memo_e_[1])
            return memo_log_[1];
        real_type result;
        if (cache_key_ && energy == *cache_key_)
        {
            result = *cache_val_;
        }
        else
        {
            result = libm::log(energy);
            if (cache_key_ && energy == slot_energy_)
            {
                *cache_key_ = energy;
                *cache_val_ = result;
            }
        }
        memo_e_[1] = memo_e_[0];
        memo_log_[1] = memo_log_[0];
        memo_e_[0] = energy;
        memo_log_[0] = result;
        return result;
    }
    GBX_FORCEINLINE ProcessGroup const& group() const { return group_; }
    GBX_FORCEINLINE MaterialRecord const& material() const
    {
        return p_.materials[material_];
    }

    //! Value grid for a process/material or nullptr
    GBX_FORCEINLINE XsGrid const* grid(int vgt, size_type ppid) const
    {
        size_type table = group_.grid_table[vgt];
        if (table == invalid_id)
            return nullptr;
        size_type gid = p_.ints[table + ppid * p_.num_materials + material_];
        if (gid == invalid_id)
            return nullptr;
        return p_.grids + gid;
    }

    //! Model applicable at an energy for a process (GridIdFinder)
    GBX_FORCEINLINE size_type find_model(size_type ppid, real_type energy) const
    {
        real_type const* grid = p_.reals + group_.model_energy[ppid];
        size_type n = group_.num_models[ppid] + 1;
        // lower_bound
        size_type lo = 0, count = n;
        while (count > 0)
        {
            size_type step = count / 2;
            size_type it = lo + step;
            if (grid[it] < energy)
            {
                lo = it + 1;
                count -= step + 1;
            }
            else
            {
                count = step;
            }
        }
        if (lo == n)
            return invalid_id;
        if (lo == 0 && energy != grid[0])
            return invalid_id;
        if (lo + 1 == n || energy != grid[lo])
            --lo;
        return p_.ints[group_.model_ids[ppid] + lo];
    }

    //! Hardwired on-the-fly model for this process/energy, or invalid
    GBX_FORCEINLINE size_type hardwired_model(size_type ppid,
                                              real_type energy) const
    {
        size_type process = group_.process[ppid];
        if ((process == p_.photoelectric_process
             && energy < real_type(p_.photoelectric_table_thresh))
            || process == p_.annihilation_process)
        {
            return this->find_model(ppid, energy);
        }
        return invalid_id;
    }

    GBX_FORCEINLINE real_type calc_xs(size_type ppid, real_type energy) const
    {
        real_type result = 0;
        size_type model = this->hardwired_model(ppid, energy);
        if (model != invalid_id)
        {
            if (model == p_.livermore_model)
                result = livermore_pe_macro_xs(p_, this->material(), energy);
            else if (model == p_.eplusgg_model)
                result = eplusgg_macro_xs(p_, this->material(), energy);
        }
        else if (XsGrid const* g = this->grid(vgt_macro_xs, ppid))
        {
            result = calc_grid_xs(p_, *g, energy, this->log_energy(energy));
        }
        return result;
    }

    GBX_FORCEINLINE real_type calc_max_xs(size_type ppid, real_type energy) const
    {
        real_type energy_max_xs
            = p_.reals[group_.energy_max_xs[ppid] + material_];
        real_type energy_xi = energy * real_type(p_.min_eprime_over_e);
        if (energy_max_xs >= energy_xi && energy_max_xs < energy)
        {
            return this->calc_xs(ppid, energy_max_xs);
        }
        return max_of(this->calc_xs(ppid, energy),
                      this->calc_xs(ppid, energy_xi));
    }

    //! Step from range (src/celeritas/phys/PhysicsTrackView.hh range_to_step)
    GBX_FORCEINLINE real_type range_to_step(real_type range) const
    {
        real_type const rho = p_.min_range;
        constexpr real_type sqrt_tol = sizeof(real_type) == 8 ? 1.0e-6 : 1.0e-3f;
        if (range < rho * (1 + sqrt_tol))
            return range;
        real_type const alpha = p_.max_step_over_range;
        return alpha * range + rho * (1 - alpha) * (2 - rho / range);
    }

  private:
    ParamsData const& p_;
    ProcessGroup const& group_;
    size_type particle_;
    size_type material_;
    // log_energy's remembered arguments (NaN: none yet) and results
    mutable real_type memo_e_[2]{real_type(NAN), real_type(NAN)};
    mutable real_type memo_log_[2]{0, 0};
    //! Per-slot cache of log(energy) (FP64 build; null otherwise)
    real_type* cache_key_{nullptr};
    real_type* cache_val_{nullptr};
    real_type slot_energy_{0};
};

//---------------------------------------------------------------------------//
// Particle kinematics (src/celeritas/phys/ParticleTrackView.hh)
//---------------------------------------------------------------------------//
GBX_FORCEINLINE real_type beta_sq(real_type mass, real_type energy)
{
    real_type inv_gamma = mass / (energy + mass);
    return 1 - ipow<2>(inv_gamma);
}
GBX_FORCEINLINE real_type momentum_sq(real_type mass, real_type energy)
{
    return ipow<2>(energy) + 2 * mass * energy;
}

//---------------------------------------------------------------------------//
// Energy loss fluctuations (Urban model)
//---------------------------------------------------------------------------//
template<class G>
GBX_FORCEINLINE real_type sample_fast_urban(real_type mean,
                                            real_type stddev,
                                            G& rng)
{
    if (stddev <= 4 * mean)
    {
        // EnergyLossGaussianDistribution: normal truncated to (0, 2 mean]
        real_type max_loss = 2 * mean;
        NormalDistribution<real_type> sample_normal(mean, stddev);
        real_type result;
        do
        {
            result = sample_normal(rng);
        } while (result <= 0 || result > max_loss);
        return result;
    }
    return UniformRealDistribution<real_type>(0, 2 * mean)(rng);
}

//! Sample the Urban energy loss given the helper's precomputed quantities
template<class G>
GBX_FUNCTION real_type sample_urban_eloss(UrbanFluctRecord const& params,
                                          MaterialRecord const& mat,
                                          real_type unscaled_mean_loss,
                                          real_type max_energy,
                                          real_type two_mebsgs,
                                          real_type beta_sq_val,
                                          G& rng)
{
    constexpr real_type rate = 0.56;
    constexpr real_type max_collisions = 8;
    constexpr real_type exc_thresh = 42;
    constexpr real_type e_0 = 1e-5;  // ionization energy [MeV]
    constexpr real_type fwhm_min_energy = 1e-3;

    real_type const loss_scaling
        = real_type(0.5) * min_of(fwhm_min_energy / max_energy, real_type(1))
          + real_type(1);
    real_type const mean_loss = unscaled_mean_loss / loss_scaling;

    real_type binding_energy[2] = {real_type(params.binding_energy[0]),
                                   real_type(params.binding_energy[1])};
    real_type xs_exc[2] = {0, 0};
    if (max_energy > real_type(mat.mean_exc_energy))
    {
        real_type const w = libm::log(two_mebsgs) - beta_sq_val;
        real_type const w_0 = mat.log_mean_exc_energy;
        if (w > w_0)
        {
            if (w > real_type(params.log_binding_energy[1]))
            {
                real_type const c = mean_loss * (1 - rate) / (w - w_0);
                for (int i = 0; i < 2; ++i)
                {
                    xs_exc[i] = c * real_type(params.oscillator_strength[i])
                                * (w - real_type(params.log_binding_energy[i]))
                                / real_type(params.binding_energy[i]);
                }
            }
            else
            {
                xs_exc[0] = mean_loss * (1 - rate)
                            / real_type(params.binding_energy[0]);
            }
            real_type scaling = 4;
            if (xs_exc[0] < exc_thresh)
            {
                scaling = real_type(0.5)
                          + (scaling - real_type(0.5))
                                * std::sqrt(xs_exc[0] / exc_thresh);
            }
            binding_energy[0] *= scaling;
            xs_exc[0] /= scaling;
        }
    }
    real_type xs_ion = mean_loss * (max_energy - e_0)
                       / (max_energy * e_0 * libm::log(max_energy / e_0));
    if (xs_exc[0] + xs_exc[1] > 0)
    {
        xs_ion *= rate;
    }

    // Excitation loss
    real_type exc_result = 0;
    {
        real_type mean = 0;
        real_type variance = 0;
        for (int i = 0; i < 2; ++i)
        {
            if (xs_exc[i] > max_collisions)
            {
                mean += xs_exc[i] * binding_energy[i];
                variance += xs_exc[i] * ipow<2>(binding_energy[i]);
            }
            else if (xs_exc[i] > 0)
            {
                unsigned int n = sample_poisson<real_type>(xs_exc[i], rng);
                if (n > 0)
                {
                    UniformRealDistribution<real_type> sample_fraction(
                        real_type(n - 1), real_type(n + 1));
                    exc_result += sample_fraction(rng) * binding_energy[i];
                }
            }
        }
        if (variance > 0)
        {
            exc_result += sample_fast_urban(mean, std::sqrt(variance), rng);
        }
    }

    // Ionization loss
    real_type ion_result = 0;
    {
        real_type const energy_ratio = max_energy / e_0;
        real_type alpha = 1;
        real_type mean_num_coll = 0;
        if (xs_ion > max_collisions)
        {
            alpha = (xs_ion + max_collisions) * energy_ratio
                    / (max_collisions * energy_ratio + xs_ion);
            real_type const mean_loss_coll = alpha * libm::log(alpha) / (alpha - 1);
            mean_num_coll = xs_ion * energy_ratio * (alpha - 1)
                            / ((energy_ratio - 1) * alpha);
            real_type const mean = mean_num_coll * mean_loss_coll * e_0;
            real_type const stddev
                = e_0 * std::sqrt(xs_ion * (alpha - ipow<2>(mean_loss_coll)));
            ion_result += sample_fast_urban(mean, stddev, rng);
        }
        if (xs_ion > 0 && energy_ratio > alpha)
        {
            real_type const lambda = xs_ion - mean_num_coll;
            UniformRealDistribution<real_type> sample_fraction(
                alpha / energy_ratio, 1);
            for (auto n = sample_poisson<real_type>(lambda, rng); n > 0; --n)
            {
                ion_result += alpha * e_0 / sample_fraction(rng);
            }
        }
    }
    return loss_scaling * (exc_result + ion_result);
}

}  // namespace gbx
