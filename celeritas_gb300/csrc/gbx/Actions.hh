// Per-slot bodies of the step-loop actions. Each function advances one track
// slot through one action; the CUDA kernels launch them one thread per slot
// and the host test driver calls them in a loop over slots.
//
// Action semantics follow the reference's executors:
//   pre-step          src/celeritas/phys/detail/PreStepExecutor.hh:46-115
//   along-step        src/celeritas/global/alongstep/AlongStepGeneralLinearAction.cc
//                     (PropagationApplier, TimeUpdater, ElossApplier with
//                     FluctELoss/MeanELoss, TrackUpdater in detail/)
//   discrete select   src/celeritas/phys/detail/DiscreteSelectExecutor.hh:38-63
//   interactions      src/celeritas/phys/InteractionApplier.hh:105-171 with the
//                     model executors in src/celeritas/em/executor/
//   geo-boundary      src/celeritas/geo/detail/BoundaryExecutor.hh:33-80
//   tracking-cut      src/celeritas/phys/detail/TrackingCutExecutor.hh
//   step gather/calo  src/celeritas/user/detail/StepGatherExecutor.hh and
//                     SimpleCaloExecutor.hh:48-67
#pragma once

#include "Field.hh"
#include "Geometry.hh"
#include "Interactors.hh"
#include "Msc.hh"

namespace gbx
{
//---------------------------------------------------------------------------//
// Small accessors
//---------------------------------------------------------------------------//
GBX_FORCEINLINE RVec3 load_dir(StateData const& s, size_type slot)
{
    return {real_type(s.dir[0][slot]),
            real_type(s.dir[1][slot]),
            real_type(s.dir[2][slot])};
}

GBX_FORCEINLINE real_type cutoff_energy(ParamsData const& p,
                                        size_type material,
                                        size_type particle)
{
    return p.cutoff_energy[material * p.num_particles + particle];
}

//! Mark a track as failed (CoreTrackView::apply_errored)
GBX_FORCEINLINE void apply_errored(ParamsData const& p,
                                   StateData const& s,
                                   size_type slot)
{
    s.status[slot] = status_errored;
    s.along_step_action[slot] = invalid_id;
    s.post_step_action[slot] = p.action_tracking_cut;
}

//---------------------------------------------------------------------------//
// pre-step
//---------------------------------------------------------------------------//
GBX_FUNCTION void pre_step(ParamsData const& p, StateData const& s, size_type slot)
{
    std::uint8_t status = s.status[slot];
    if (status == status_inactive)
    {
        s.step_length[slot] = INFINITY;
        s.post_step_action[slot] = invalid_id;
        s.along_step_action[slot] = invalid_id;
        return;
    }
    s.energy_deposition[slot] = 0;
    s.secondaries_offset[slot] = 0;
    s.secondaries_count[slot] = 0;
    s.element[slot] = invalid_id;
    if (status == status_errored)
        return;
    s.status[slot] = status_alive;

    if (!(s.interaction_mfp[slot] > 0))
    {
        XorwowEngine rng(s.rng, slot);
        s.interaction_mfp[slot] = sample_exponential<real_type>(rng);
    }

    size_type const pid = s.particle_id[slot];
    size_type const mid = s.material[slot];
    real_type const energy = s.energy[slot];
    PhysicsTrack phys(p, pid, mid, s, slot);

    // calc_physics_step_limit
    real_type total_macro_xs = 0;
    for (size_type ppid = 0; ppid < phys.num_processes(); ++ppid)
    {
        real_type process_xs;
        if (phys.group().use_integral[ppid])
            process_xs = phys.calc_max_xs(ppid, energy);
        else
            process_xs = phys.calc_xs(ppid, energy);
        total_macro_xs += process_xs;
        s.per_process_xs[ppid][slot] = process_xs;
    }
    s.macro_xs[slot] = total_macro_xs;

    real_type step;
    size_type action = p.action_discrete;
    if (energy == 0)
    {
        step = 0;
    }
    else
    {
        step = s.interaction_mfp[slot] / total_macro_xs;
        size_type const eloss = phys.group().eloss_process;
        if (eloss != invalid_id)
        {
            XsGrid const* g = phys.grid(vgt_range, eloss);
            real_type range = calc_range(p, *g, energy, phys.log_energy(energy));
            s.dedx_range[slot] = range;
            real_type eloss_step = phys.range_to_step(range);
            if (eloss_step <= step)
            {
                step = eloss_step;
                action = p.action_range;
            }
        }
        else if (phys.num_processes() == 0)
        {
            action = invalid_id;
        }
    }
    if constexpr (sizeof(real_type) < sizeof(double))
    {
        // FP32: a near-vacuum gives physics steps of ~1e23 cm whose products
        // overflow FP32 in the multiple-scattering and field-integration
        // arithmetic; any step above 1e10 cm is limited by the geometry
        // long before it ends, so the cap changes no step that is taken
        step = min_of(step, real_type(1e10));
    }
    s.step_length[slot] = step;
    s.post_step_action[slot] = action;
    s.along_step_action[slot] = (p.particles[pid].charge == 0)
                                    ? p.action_along_step_neutral
                                    : p.action_along_step;
}

//---------------------------------------------------------------------------//
// along-step (linear propagation, energy loss, track update)
//---------------------------------------------------------------------------//
//! Mean energy loss over a step (calc_mean_energy_loss)
GBX_FORCEINLINE real_type calc_mean_eloss(ParamsData const& p,
                                          StateData const& s,
                                          PhysicsTrack const& phys,
                                          size_type slot,
                                          real_type pre_energy,
                                          real_type step)
{
    size_type const ppid = phys.group().eloss_process;
    XsGrid const* dedx = phys.grid(vgt_energy_loss, ppid);
    real_type eloss = step * calc_grid_xs(p, *dedx, pre_energy, phys.log_energy(pre_energy));
    if (eloss >= pre_energy * real_type(p.linear_loss_limit))
    {
        XsGrid const* rg = phys.grid(vgt_range, ppid);
        real_type range = s.dedx_range[slot];
        if (step == range)
            return pre_energy;
        eloss = pre_energy - calc_inverse_range(p, *rg, range - step);
    }
    return eloss;
}

//! Fluctuating (or mean) energy loss: FluctELoss::calc_eloss
template<class G>
GBX_FUNCTION real_type calc_eloss(ParamsData const& p,
                                  StateData const& s,
                                  PhysicsTrack const& phys,
                                  size_type slot,
                                  real_type step,
                                  bool apply_cut,
                                  G& rng)
{
    real_type const energy = s.energy[slot];
    real_type const lowest = p.lowest_electron_energy;
    if (apply_cut && energy < lowest)
        return energy;
    real_type eloss = calc_mean_eloss(p, s, phys, slot, energy, step);
    if (p.enable_fluct && eloss < energy)
    {
        // EnergyLossHelper (src/celeritas/em/distribution/EnergyLossHelper.hh)
        size_type const pid = s.particle_id[slot];
        size_type const mid = s.material[slot];
        real_type const mean_loss = eloss;
        if (!(mean_loss < real_type(1e-5)))
        {
            real_type const mass = p.particles[pid].mass;
            real_type const electron_mass = p.particles[p.electron_id].mass;
            real_type const gamma = 1 + energy / mass;
            real_type const bsq = beta_sq(mass, energy);
            real_type const two_mebsgs = 2 * electron_mass * bsq * ipow<2>(gamma);
            real_type max_energy_transfer;
            if (pid == p.electron_id)
            {
                max_energy_transfer = real_type(0.5) * energy;
            }
            else
            {
                real_type mass_ratio = electron_mass / mass;
                max_energy_transfer
                    = two_mebsgs / (1 + mass_ratio * (2 * gamma + mass_ratio));
            }
            real_type const max_energy = min_of(
                real_type(cutoff_energy(p, mid, p.electron_id)), max_energy_transfer);
            if (max_energy > real_type(1e-5))
            {
                // e+/e- have mass ratio 1: always the Urban model
                eloss = sample_urban_eloss(p.fluct[mid],
                                           p.materials[mid],
                                           mean_loss,
                                           max_energy,
                                           two_mebsgs,
                                           bsq,
                                           rng);
            }
        }
        if (eloss >= energy)
        {
            eloss = apply_cut ? energy : mean_loss;
        }
    }
    if (apply_cut && (energy - eloss <= lowest))
        return energy;
    return eloss;
}

//! Which along-step actions a compiled along-step function handles: both
//! (selected per slot), or only one, so that the neutral instance carries
//! none of the charged-particle code and its registers
enum class AlongKind
{
    any,
    charged,
    neutral,
};

//! Start of the along-step: track and action checks and the multiple-
//! scattering step limit. Returns false if this function kind does not
//! handle the slot (nothing was done).
template<AlongKind K>
GBX_FUNCTION bool along_prologue(ParamsData const& p,
                                 StateData const& s,
                                 size_type slot,
                                 bool* charged,
                                 double* start_safety = nullptr)
{
    size_type const along = s.along_step_action[slot];
    if (!is_track_valid(s.status[slot]))
        return false;
    if (K != AlongKind::neutral && along == p.action_along_step)
    {
    }
    else if (K != AlongKind::charged && along == p.action_along_step_neutral)
    {
    }
    else
    {
        return false;
    }
    *charged = (K == AlongKind::charged)
               || (K == AlongKind::any && along == p.action_along_step);

    // MscStepLimitApplier
    double safety = 0;
    if (*charged && p.msc.enabled)
    {
        XorwowEngine rng(s.rng, slot);
        safety = msc_limit_step(p, s, slot, rng);
    }
    if (start_safety)
        *start_safety = safety;
    return true;
}

//! Set up the uniform-field propagation of a charged slot over its step
GBX_FUNCTION void field_setup(ParamsData const& p,
                              StateData const& s,
                              size_type slot,
                              GeoTrackView& geo,
                              FieldPropagation* fp,
                              double start_safety)
{
    size_type const pid = s.particle_id[slot];
    real_type const mass = p.particles[pid].mass;
    real_type const energy = s.energy[slot];
    double const momentum = std::sqrt(double(momentum_sq(mass, energy)));
    UniformFieldEquation rhs;
    rhs.field = {p.field[0], p.field[1], p.field[2]};
    rhs.map = p.has_rzmap ? p.rzmap : nullptr;
    rhs.coeffi = (p.particles[pid].charge * detail::e_electron)
                 / (1 * (detail::mev_value / constants::c_light));
    fp->set_rhs(rhs);
    fp->init(geo, momentum, s.step_length[slot], start_safety);
}

//! Step limit and looping bookkeeping after a field propagation
GBX_FUNCTION void field_result(ParamsData const& p,
                               StateData const& s,
                               size_type slot,
                               Propagation const& prop)
{
    size_type const pid = s.particle_id[slot];
    real_type const energy = s.energy[slot];
    double const step_length = s.step_length[slot];
    // update_looping. With reentrant_looping, a step that ends on a boundary
    // the track re-enters at once (its direction at the boundary points back
    // into the volume it came from) is no progress and keeps the count.
    bool const reentry = p.reentrant_looping && prop.boundary
                         && s.boundary[slot] == boundary_reentrant;
    if (prop.looping)
        ++s.num_looping_steps[slot];
    else if (!reentry)
        s.num_looping_steps[slot] = 0;
    if (prop.looping)
    {
        s.step_length[slot] = prop.distance;
        LoopingRecord const& lr = p.looping[pid];
        size_type const max_steps = (energy < real_type(lr.threshold_energy))
                                        ? lr.max_subthreshold_steps
                                        : lr.max_steps;
        s.post_step_action[slot] = (s.num_looping_steps[slot] >= max_steps)
                                       ? p.action_tracking_cut
                                       : p.action_propagation_limit;
    }
    else if (prop.boundary)
    {
        s.step_length[slot] = prop.distance;
        s.post_step_action[slot] = p.action_boundary;
    }
    else if (prop.distance < step_length)
    {
        s.step_length[slot] = prop.distance;
        s.post_step_action[slot] = p.action_propagation_limit;
    }
}

//! Straight-line propagation over the slot's step
GBX_FUNCTION void linear_propagation(ParamsData const& p,
                                     StateData const& s,
                                     size_type slot,
                                     GeoTrackView& geo)
{
    double const step_length = s.step_length[slot];
    Propagation prop = geo.find_next_step(step_length);
    if (prop.boundary)
        geo.move_to_boundary();
    else
        geo.move_internal(step_length);
    if (prop.boundary)
    {
        s.step_length[slot] = prop.distance;
        s.post_step_action[slot] = p.action_boundary;
    }
    else if (prop.distance < step_length)
    {
        s.step_length[slot] = prop.distance;
        s.post_step_action[slot] = p.action_propagation_limit;
    }
}

//! End of the along-step after propagation: multiple-scattering
//! deflection and displacement, time, energy loss and track update
GBX_FUNCTION void along_epilogue(ParamsData const& p,
                                 StateData const& s,
                                 size_type slot,
                                 bool charged)
{
    // MscApplier
    if (charged && p.msc.enabled)
    {
        XorwowEngine rng(s.rng, slot);
        msc_apply_step(p, s, slot, rng);
    }

    // TimeUpdater
    if (s.status[slot] == status_errored)
        return;
    size_type const pid = s.particle_id[slot];
    {
        real_type const mass = p.particles[pid].mass;
        real_type const speed
            = std::sqrt(beta_sq(mass, s.energy[slot])) * real_type(constants::c_light);
        if (speed > 0)
        {
            // Time accumulates in FP64; the increment is a physics quantity
            s.time[slot] += double(real_type(s.step_length[slot]) / speed);
        }
    }

    // ElossApplier
    PhysicsTrack phys(p, pid, s.material[slot], s, slot);
    if (charged && phys.group().eloss_process != invalid_id && s.energy[slot] != 0)
    {
        real_type const step = s.step_length[slot];
        bool const apply_cut = (s.post_step_action[slot] != p.action_boundary);
        real_type deposited;
        {
            XorwowEngine rng(s.rng, slot);
            deposited = calc_eloss(p, s, phys, slot, step, apply_cut, rng);
        }
        if (deposited > 0)
        {
            s.energy_deposition[slot] += deposited;
            s.energy[slot] -= deposited;
        }
        if (s.energy[slot] == 0)
        {
            if (!phys.group().has_at_rest)
            {
                s.status[slot] = status_killed;
                s.post_step_action[slot] = p.action_range;
            }
            else
            {
                s.post_step_action[slot] = p.action_discrete;
            }
        }
    }

    // TrackUpdater
    if (s.status[slot] == status_alive)
    {
        if (s.post_step_action[slot] != p.action_discrete)
        {
            real_type mfp = s.interaction_mfp[slot]
                            - real_type(s.step_length[slot]) * s.macro_xs[slot];
            s.interaction_mfp[slot] = mfp;
        }
    }
    ++s.num_steps[slot];
}

//! The whole along-step of one slot (PropagationApplier between the MSC
//! step limit and the MSC applier, then time, energy loss, track update)
template<AlongKind K>
GBX_FUNCTION void along_step_impl(ParamsData const& p, StateData const& s, size_type slot)
{
    bool charged;
    double start_safety;
    if (!along_prologue<K>(p, s, slot, &charged, &start_safety))
        return;
    // PropagationApplier: straight line, or the uniform-field integrator for
    // charged tracks (which can loop)
    if (s.step_length[slot] != 0)
    {
        GeoTrackView geo(p.geo, s, slot);
        if (charged && p.has_field)
        {
            FieldOptions const& opt = p.field_options;
            FieldPropagation fp(opt, UniformFieldEquation{});
            field_setup(p, s, slot, geo, &fp, start_safety);
            do
            {
                fp.substep(geo);
            } while (!fp.done());
            field_result(p, s, slot, fp.finish(geo));
        }
        else
        {
            linear_propagation(p, s, slot, geo);
        }
    }
    along_epilogue(p, s, slot, charged);
}

GBX_FORCEINLINE void along_step(ParamsData const& p, StateData const& s, size_type slot)
{
    along_step_impl<AlongKind::any>(p, s, slot);
}

//---------------------------------------------------------------------------//
// discrete select
//---------------------------------------------------------------------------//
GBX_FUNCTION void discrete_select(ParamsData const& p,
                                  StateData const& s,
                                  size_type slot)
{
    if (s.post_step_action[slot] != p.action_discrete)
        return;
    s.interaction_mfp[slot] = 0;
    size_type const pid = s.particle_id[slot];
    size_type const mid = s.material[slot];
    real_type const energy = s.energy[slot];
    PhysicsTrack phys(p, pid, mid, s, slot);
    XorwowEngine rng(s.rng, slot);

    // Select the process (Selector with total = macro xs)
    size_type const nproc = phys.num_processes();
    size_type ppid = nproc - 1;
    {
        real_type accum = -s.macro_xs[slot] * generate_canonical<real_type>(rng);
        for (size_type i = 0; i + 1 < nproc; ++i)
        {
            accum += s.per_process_xs[i][slot];
            if (accum > 0)
            {
                ppid = i;
                break;
            }
        }
    }
    size_type action;
    if (phys.group().use_integral[ppid])
    {
        real_type xs = phys.calc_xs(ppid, energy);
        if (generate_canonical<real_type>(rng) * s.per_process_xs[ppid][slot] > xs)
        {
            s.post_step_action[slot] = p.action_integral_rejection;
            return;
        }
    }
    size_type const model = phys.find_model(ppid, energy);
    if (model == invalid_id)
    {
        // No model applies at this energy (possible only for a corrupted
        // track state): fail the track instead of dispatching nowhere
        apply_errored(p, s, slot);
        return;
    }
    MaterialRecord const& mat = p.materials[mid];
    if (mat.num_elements == 1)
    {
        s.element[slot] = 0;
    }
    else
    {
        // Sample the element from the model's tabulated cross-section CDF
        // (TabulatedElementSelector, src/celeritas/mat/TabulatedElementSelector.hh)
        size_type const table
            = p.ints[p.element_tables
                     + (model * p.num_particles + pid) * p.num_materials + mid];
        if (table != invalid_id)
        {
            real_type const u = generate_canonical<real_type>(rng);
            size_type i = 0;
            for (; i + 1 < mat.num_elements; ++i)
            {
                if (calc_grid_xs(
                        p, p.grids[p.ints[table + i]], energy, phys.log_energy(energy))
                    > u)
                    break;
            }
            s.element[slot] = i;
        }
    }
    action = model + p.model_to_action;
    s.post_step_action[slot] = action;
}

//---------------------------------------------------------------------------//
// Interaction application (InteractionApplier)
//---------------------------------------------------------------------------//
GBX_FUNCTION void apply_interaction(ParamsData const& p,
                                    StateData const& s,
                                    size_type slot,
                                    Interaction const& result)
{
    if (result.action == Interaction::failed)
    {
        // sim.step_limit({0, failure_action})
        if (0 < s.step_length[slot])
        {
            s.step_length[slot] = 0;
            s.post_step_action[slot] = p.action_failure;
        }
        return;
    }
    if (result.action == Interaction::unchanged)
        return;
    // In FP32 the difference of two energies can round to just below zero
    // (FP64 never reaches this branch on the reference's inputs): such a
    // particle is at rest, and one without an at-rest process ends here
    real_type energy = result.energy;
    if (energy < 0)
    {
        energy = 0;
        if (!p.process_groups[s.particle_id[slot]].has_at_rest)
            s.status[slot] = status_killed;
    }
    for (size_type i = 0; i < result.num_secondaries; ++i)
    {
        Secondary& sec = result.secondaries[i];
        if (sec.energy < 0 && sec.particle_id != invalid_id)
        {
            sec.energy = 0;
            if (!p.process_groups[sec.particle_id].has_at_rest)
                sec.particle_id = invalid_id;
        }
    }
    s.energy[slot] = energy;
    if (result.action != Interaction::absorbed)
    {
        GeoTrackView geo(p.geo, s, slot);
        geo.set_dir(to_geo_dir(result.direction));
    }
    else
    {
        s.status[slot] = status_killed;
    }
    s.energy_deposition[slot] += result.energy_deposition;
    s.secondaries_offset[slot] = result.secondaries
                                     ? static_cast<size_type>(
                                         result.secondaries - s.secondaries)
                                     : 0;
    s.secondaries_count[slot] = result.num_secondaries;
}

//! Run one model's interaction for a slot whose post-step action matches
GBX_FUNCTION void interact(ParamsData const& p,
                           StateData const& s,
                           size_type slot,
                           size_type action)
{
    if (s.post_step_action[slot] != action)
        return;
    size_type const pid = s.particle_id[slot];
    size_type const mid = s.material[slot];
    real_type const energy = s.energy[slot];
    RVec3 const dir = load_dir(s, slot);
    SecondaryAllocator allocate(s);
    Interaction result;
    {
        XorwowEngine rng(s.rng, slot);
        MaterialRecord const& mat = p.materials[mid];
        size_type const elcomp = s.element[slot];
        if ((action == p.action_bethe_heitler || action == p.action_seltzer_berger
             || action == p.action_rel_brems || action == p.action_combined_brems)
            && !(elcomp < mat.num_elements))
        {
            // Element-dependent model without a sampled element (possible
            // only for a corrupted track state)
            apply_errored(p, s, slot);
            return;
        }
        if (action == p.action_klein_nishina)
        {
            result = interact_klein_nishina(p, energy, dir, allocate, rng);
        }
        else if (action == p.action_livermore_pe)
        {
            size_type el = elcomp;
            if (el == invalid_id)
            {
                // Sample the element with on-the-fly micro cross sections
                // (ElementSelector in LivermorePEExecutor.hh:41-54)
                real_type micro[max_elements];
                real_type material_xs = 0;
                for (size_type j = 0; j < mat.num_elements; ++j)
                {
                    micro[j] = livermore_pe_micro_xs(p, mat.element[j], energy);
                    material_xs += micro[j] * mat.fraction[j];
                }
                real_type accum = -material_xs * generate_canonical<real_type>(rng);
                el = 0;
                for (; el + 1 < mat.num_elements; ++el)
                {
                    accum += mat.fraction[el] * micro[el];
                    if (accum > 0)
                        break;
                }
                s.element[slot] = el;
            }
            result = interact_livermore_pe(
                p, mat.element[el], energy, dir, allocate, rng);
        }
        else if (action == p.action_bethe_heitler)
        {
            result = interact_bethe_heitler(
                p, p.elements[mat.element[elcomp]], energy, dir, allocate, rng);
        }
        else if (action == p.action_seltzer_berger
                 || (action == p.action_combined_brems
                     && energy < seltzer_berger_upper_limit))
        {
            // CombinedBremInteractor (CombinedBremInteractor.hh:129-160)
            // samples with Seltzer-Berger below 1 GeV and the relativistic
            // sampler above, the same final state after either
            result = interact_seltzer_berger(p,
                                             mat.element[elcomp],
                                             mat,
                                             pid == p.electron_id,
                                             real_type(p.particles[pid].mass),
                                             energy,
                                             dir,
                                             cutoff_energy(p, mid, p.gamma_id),
                                             allocate,
                                             rng);
        }
        else if (action == p.action_rel_brems || action == p.action_combined_brems)
        {
            result = interact_relativistic_brems(p,
                                                 mat.element[elcomp],
                                                 mat,
                                                 real_type(p.particles[pid].mass),
                                                 energy,
                                                 dir,
                                                 cutoff_energy(p, mid, p.gamma_id),
                                                 allocate,
                                                 rng);
        }
        else if (action == p.action_moller_bhabha)
        {
            result = interact_moller_bhabha(p,
                                            pid == p.electron_id,
                                            energy,
                                            dir,
                                            cutoff_energy(p, mid, p.electron_id),
                                            allocate,
                                            rng);
        }
        else if (action == p.action_eplusgg)
        {
            result = interact_eplusgg(p, energy, dir, allocate, rng);
        }
        else
        {
            return;
        }
    }
    apply_interaction(p, s, slot, result);
}

//---------------------------------------------------------------------------//
// geo-boundary and tracking-cut
//---------------------------------------------------------------------------//
GBX_FUNCTION void boundary_cross(ParamsData const& p,
                                 StateData const& s,
                                 size_type slot)
{
    if (s.post_step_action[slot] != p.action_boundary)
        return;
    GeoTrackView geo(p.geo, s, slot);
    geo.cross_boundary();
    if (geo.failed())
    {
        apply_errored(p, s, slot);
        return;
    }
    if (!geo.is_outside())
    {
        size_type matid = p.geo.volume_material[geo.volume()];
        if (matid == invalid_id)
        {
            apply_errored(p, s, slot);
            return;
        }
        s.material[slot] = matid;
    }
    else
    {
        s.status[slot] = status_killed;
    }
}

GBX_FUNCTION void tracking_cut(ParamsData const& p,
                               StateData const& s,
                               size_type slot)
{
    if (s.post_step_action[slot] != p.action_tracking_cut)
        return;
    size_type const pid = s.particle_id[slot];
    real_type deposited = s.energy[slot];
    if (p.particles[pid].is_antiparticle)
    {
        deposited += 2 * real_type(p.particles[pid].mass);
    }
    s.energy_deposition[slot] += deposited;
    s.energy[slot] -= s.energy[slot];
    s.status[slot] = status_killed;
}

//---------------------------------------------------------------------------//
// Step gathering and calorimeter tally
//---------------------------------------------------------------------------//
//! Record the detector of the pre-step volume and, when hits are collected,
//! the pre-step point of a slot in a detector (StepGatherExecutor<pre>,
//! src/celeritas/user/detail/StepGatherExecutor.hh:52-150)
GBX_FUNCTION void gather_pre(ParamsData const& p, StateData const& s, size_type slot)
{
    if (s.status[slot] == status_inactive)
    {
        s.detector[slot] = invalid_id;
        return;
    }
    size_type vol = s.volume[slot];
    size_type const det = p.geo.volume_detector[vol];
    s.detector[slot] = det;
    if (det == invalid_id)
        return;
    if (s.pre_time)
        s.pre_time[slot] = s.time[slot];
    if (s.pre_pos)
    {
        for (int i = 0; i < 3; ++i)
            s.pre_pos[3 * std::size_t(slot) + i] = s.pos[i][slot];
    }
    if (s.pre_dir)
    {
        for (int i = 0; i < 3; ++i)
            s.pre_dir[3 * std::size_t(slot) + i] = s.dir[i][slot];
    }
    if (s.pre_energy)
        s.pre_energy[slot] = double(s.energy[slot]);
}

//! Whether a slot's step is a hit: an active track that started the step in
//! a detector volume and, with the filter, deposited energy
//! (StepGatherExecutor<post>; DetectorSteps keeps the slots whose detector
//! is still set, src/celeritas/user/DetectorSteps.cc)
GBX_FUNCTION bool has_step_hit(StateData const& s, StepHitsRef const& h, size_type slot)
{
    if (s.status[slot] == status_inactive || s.detector[slot] == invalid_id)
        return false;
    return !(h.nonzero_energy_deposition && s.energy_deposition[slot] == 0);
}

//! Write a slot's hit as record 'i' of the step output: the selected
//! post-step data gathered from the track now, the pre-step point gathered
//! at pre-step; the particle as the reference's ParticleId
GBX_FUNCTION void write_step_hit(ParamsData const& p,
                                 StateData const& s,
                                 StepHitsRef const& h,
                                 size_type slot,
                                 size_type i,
                                 size_type step)
{
    std::size_t const i3 = 3 * std::size_t(i);
    std::size_t const s3 = 3 * std::size_t(slot);
    h.step[i] = step;
    h.detector[i] = s.detector[slot];
    h.track_id[i] = s.track_id[slot];
    if (h.event_id)
        h.event_id[i] = s.event_id[slot];
    if (h.parent_id)
        h.parent_id[i] = s.parent_id[slot];
    if (h.track_step_count)
        h.track_step_count[i] = s.num_steps[slot];
    if (h.particle)
        h.particle[i] = p.particles[s.particle_id[slot]].ref_id;
    if (h.step_length)
        h.step_length[i] = s.step_length[slot];
    if (h.energy_deposition)
        h.energy_deposition[i] = double(s.energy_deposition[slot]);
    if (h.pre_time)
        h.pre_time[i] = s.pre_time[slot];
    if (h.pre_energy)
        h.pre_energy[i] = s.pre_energy[slot];
    for (int k = 0; k < 3; ++k)
    {
        if (h.pre_pos)
            h.pre_pos[i3 + k] = s.pre_pos[s3 + k];
        if (h.pre_dir)
            h.pre_dir[i3 + k] = s.pre_dir[s3 + k];
        if (h.post_pos)
            h.post_pos[i3 + k] = s.pos[k][slot];
        if (h.post_dir)
            h.post_dir[i3 + k] = s.dir[k][slot];
    }
    if (h.post_time)
        h.post_time[i] = s.time[slot];
    if (h.post_energy)
        h.post_energy[i] = double(s.energy[slot]);
}

}  // namespace gbx
