// CPU restatement of the reference's host stepping loop, used (1) to check
// the per-slot action code of the GB300 path against the reference itself on
// the CPU, and (2) as the timed CPU baseline on machines where the reference
// cannot be built.
//
// The loop follows Stepper<MemSpace::host>::operator()
// (src/celeritas/global/Stepper.cc:125-168) and ActionSequence::step
// (src/celeritas/global/ActionSequence.cc:77-138): actions run in
// (StepActionOrder, ActionId) order, each over all track slots in slot order.
// The per-slot bodies are the GB300 path's host+device action functions
// (celeritas_gb300/csrc/gbx/Actions.hh, TrackInit.hh) compiled for the host;
// the global steps (vacancy compaction, secondary-count scan, initializer
// bookkeeping) are restated here sequentially
// (src/celeritas/track/detail/TrackInitAlgorithms.cc).
//
// This is test and baseline infrastructure, never the shipped GB300 path.
//
// Usage:
//   port_stepper run <physics.txt> calo <primaries.txt> <slots> <seed>
//                    [--steps N] [--quiet] [--hits]
//   port_stepper bench <physics.txt> <geometry> <primaries.txt> <slots> <seed>
//                    [--threads T] [--event-tallies FILE] [physics options]
//   port_stepper interact|along <physics.txt> <geometry> <inputs.txt> <seed>
//                    [physics options]
//   port_stepper libm <exp|log|sin|cos|tanh|log1p|expm1|cbrt> < hex doubles
#include <algorithm>
#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../celeritas_gb300/csrc/gbx/TrackInit.hh"
#include "../../celeritas_gb300/csrc/host/HostParams.hh"
#include "../../celeritas_gb300/csrc/host/HostState.hh"

using namespace gbx;

namespace
{
struct StepCounts
{
    size_type generated{0};
    size_type queued{0};
    size_type active{0};
    size_type alive{0};
    explicit operator bool() const { return queued > 0 || alive > 0; }
};

class PortStepper
{
  public:
    PortStepper(HostParams const& hp,
                size_type num_slots,
                unsigned int seed,
                size_type max_events)
        : params_(make_host_view(hp))
        , state_(num_slots,
                 std::max<size_type>(1u << 20, 4 * num_slots),
                 max_events,
                 static_cast<size_type>(hp.scalars.secondary_stack_factor
                                        * num_slots),
                 hp.scalars.num_detectors,
                 seed)
        , action_labels_(hp.action_labels)
        , seed_(seed)
    {
    }

    //! Stepper::reseed: every slot's XORWOW state from the seed, advanced
    //! event * size + slot subsequences; per-event track IDs restart
    void reseed(unsigned long long event_id)
    {
        StateData s = state_.view();
        for (size_type i = 0; i < s.size; ++i)
        {
            reseed_xorwow_slot(
                s.rng, params_.rng_jump + 32 * 5, seed_, event_id * s.size + i, i);
        }
        std::fill(state_.track_counters.begin(), state_.track_counters.end(), 0);
    }

    //! XORWOW words of slot i: five xor words, then the Weyl word
    std::array<std::uint32_t, 6> rng_words(size_type i)
    {
        StateData s = state_.view();
        return {s.rng.s[0][i], s.rng.s[1][i], s.rng.s[2][i],
                s.rng.s[3][i], s.rng.s[4][i], s.rng.weyl[i]};
    }

    StepCounts operator()(std::vector<TrackInitializer> const& primaries)
    {
        state_.primaries = primaries;
        return this->step(true);
    }
    StepCounts operator()() { return this->step(false); }

    //! Insert primaries and run the first actions of a step (through
    //! pre-step), leaving every track ready for its step-limit action
    void prepare(std::vector<TrackInitializer> const& primaries)
    {
        state_.primaries = primaries;
        this->begin_step(true);
    }
    StateData view() { return state_.view(); }
    ParamsData const& params() const { return params_; }
    std::vector<std::string> const& action_labels() const { return action_labels_; }

    std::vector<double> const& edep() const { return state_.calo_edep; }

    //! Print every step's hits (all step data, steps without deposition
    //! dropped) as 'hit' lines
    void enable_hits()
    {
        std::size_t const n = state_.size;
        state_.pre_time.assign(n, 0);
        state_.pre_pos.assign(3 * n, 0);
        state_.pre_dir.assign(3 * n, 0);
        state_.pre_energy.assign(n, 0);
        for (auto* v : {&hb_.step, &hb_.detector, &hb_.track_id, &hb_.event_id,
                        &hb_.parent_id, &hb_.track_step_count, &hb_.particle})
            v->assign(n, 0);
        for (auto* v : {&hb_.step_length, &hb_.energy_deposition, &hb_.pre_time,
                        &hb_.pre_energy, &hb_.post_time, &hb_.post_energy})
            v->assign(n, 0);
        for (auto* v : {&hb_.pre_pos, &hb_.pre_dir, &hb_.post_pos, &hb_.post_dir})
            v->assign(3 * n, 0);
        hits_.capacity = state_.size;
        hits_.selection = step_select_all;
        hits_.nonzero_energy_deposition = true;
        hits_.step = hb_.step.data();
        hits_.detector = hb_.detector.data();
        hits_.track_id = hb_.track_id.data();
        hits_.event_id = hb_.event_id.data();
        hits_.parent_id = hb_.parent_id.data();
        hits_.track_step_count = hb_.track_step_count.data();
        hits_.particle = hb_.particle.data();
        hits_.step_length = hb_.step_length.data();
        hits_.energy_deposition = hb_.energy_deposition.data();
        hits_.pre_time = hb_.pre_time.data();
        hits_.pre_pos = hb_.pre_pos.data();
        hits_.pre_dir = hb_.pre_dir.data();
        hits_.pre_energy = hb_.pre_energy.data();
        hits_.post_time = hb_.post_time.data();
        hits_.post_pos = hb_.post_pos.data();
        hits_.post_dir = hb_.post_dir.data();
        hits_.post_energy = hb_.post_energy.data();
    }

    //! Print the state of every non-inactive slot
    void trace(size_type iter) const
    {
        HostState const& s = state_;
        for (size_type i = 0; i < s.size; ++i)
        {
            if (s.status[i] == status_inactive)
                continue;
            std::printf("trace %u %u st=%d pid=%u E=%.17g pos=(%.17g,%.17g,%.17g) "
                        "dir=(%.17g,%.17g,%.17g) vol=%u act=%d len=%.17g mfp=%.17g "
                        "edep=%.17g nsec=%u\n",
                        iter,
                        i,
                        int(s.status[i]),
                        s.particle_id[i],
                        double(s.energy[i]),
                        s.pos[0][i],
                        s.pos[1][i],
                        s.pos[2][i],
                        s.dir[0][i],
                        s.dir[1][i],
                        s.dir[2][i],
                        s.volume[i],
                        int(s.post_step_action[i]),
                        s.step_length[i],
                        double(s.interaction_mfp[i]),
                        double(s.energy_deposition[i]),
                        s.secondaries_count[i]);
        }
    }

  private:
    ParamsData params_;
    HostState state_;
    std::vector<std::string> action_labels_;
    unsigned int seed_;
    unsigned int iteration_{0};
    struct HitBuffers
    {
        std::vector<size_type> step, detector, track_id, event_id, parent_id,
            track_step_count, particle;
        std::vector<double> step_length, energy_deposition, pre_time, pre_pos,
            pre_dir, pre_energy, post_time, post_pos, post_dir, post_energy;
    } hb_;
    StepHitsRef hits_;

    void print_hits(size_type count) const
    {
        StepHitsRef const& h = hits_;
        for (size_type i = 0; i < count; ++i)
        {
            std::printf(
                "hit %u %u %u %u %u %u %u %.17g %.17g %.17g %.17g %.17g %.17g "
                "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g "
                "%.17g %.17g\n",
                h.step[i], h.detector[i], h.track_id[i], h.event_id[i],
                h.parent_id[i], h.track_step_count[i], h.particle[i],
                h.step_length[i], h.energy_deposition[i], h.pre_time[i],
                h.pre_pos[3 * i], h.pre_pos[3 * i + 1], h.pre_pos[3 * i + 2],
                h.pre_dir[3 * i], h.pre_dir[3 * i + 1], h.pre_dir[3 * i + 2],
                h.pre_energy[i], h.post_time[i], h.post_pos[3 * i],
                h.post_pos[3 * i + 1], h.post_pos[3 * i + 2], h.post_dir[3 * i],
                h.post_dir[3 * i + 1], h.post_dir[3 * i + 2], h.post_energy[i]);
        }
    }

    //! The actions of a step up to and including pre-step:
    //! extend-from-primaries, initialize-tracks, pre-step. Returns the
    //! number of active tracks.
    size_type begin_step(bool with_primaries)
    {
        ParamsData const& p = params_;
        StateData s = state_.view();
        Counters& c = state_.counters;
        size_type const n = s.size;
        c.num_generated = 0;

        // extend-from-primaries (generate)
        if (with_primaries)
        {
            size_type np = static_cast<size_type>(state_.primaries.size());
            c.num_initializers += np;
            if (c.num_initializers > s.initializer_capacity)
                throw std::runtime_error("initializer capacity exceeded");
            for (size_type i = 0; i < np; ++i)
                process_primary(s, c.num_initializers, np, i);
            c.num_generated += np;
            std::fill(state_.parents.begin(), state_.parents.end(), invalid_id);
        }
        // initialize-tracks (start)
        {
            size_type num_new = std::min(c.num_vacancies, c.num_initializers);
            if (partitions_by_charge(p.track_order))
            {
                // InitializeTracksAction with TrackOrder init_charge: the
                // last num_new initializers' offsets, neutral ones first in
                // a stable partition, then the initialization, then the
                // parent slots cleared
                size_type* idx = s.init_indices;
                for (size_type i = 0; i < num_new; ++i)
                    idx[i] = i;
                TrackInitializer const* stencil
                    = s.initializers + c.num_initializers - num_new;
                std::stable_partition(idx, idx + num_new, [&](size_type i) {
                    return is_neutral(p, stencil[i]);
                });
                for (size_type i = 0; i < num_new; ++i)
                    init_track_charge_partitioned(p, s, c, num_new, i);
            }
            else
            {
                for (size_type i = 0; i < num_new; ++i)
                    init_track(p, s, c, i);
            }
            c.num_initializers -= num_new;
            c.num_vacancies -= num_new;
            c.num_active = n - c.num_vacancies;
            if (partitions_by_charge(p.track_order))
                std::fill(state_.parents.begin(), state_.parents.end(), invalid_id);
        }
        // pre-step (pre): thread 0 clears the secondary stack
        c.secondary_stack_size = 0;
        for (size_type i = 0; i < n; ++i)
            pre_step(p, s, i);
        return c.num_active;
    }

    StepCounts step(bool with_primaries)
    {
        ParamsData const& p = params_;
        StateData s = state_.view();
        Counters& c = state_.counters;
        size_type const n = s.size;
        size_type const active = this->begin_step(with_primaries);
        // step-gather-pre (user_pre)
        for (size_type i = 0; i < n; ++i)
            gather_pre(p, s, i);
        // along-step-general-linear, along-step-neutral (along)
        for (size_type i = 0; i < n; ++i)
            along_step(p, s, i);
        // physics-discrete-select (pre_post)
        for (size_type i = 0; i < n; ++i)
            discrete_select(p, s, i);
        // models (post), in action-ID order
        for (size_type a = p.model_to_action; a < p.model_to_action + p.num_models;
             ++a)
        {
            for (size_type i = 0; i < n; ++i)
                interact(p, s, i, a);
        }
        for (size_type i = 0; i < n; ++i)
            boundary_cross(p, s, i);
        for (size_type i = 0; i < n; ++i)
            tracking_cut(p, s, i);
        // step-gather-post -> calorimeter tally (user_post)
        for (size_type i = 0; i < n; ++i)
        {
            if (s.status[i] == status_inactive)
                continue;
            size_type det = s.detector[i];
            if (det != invalid_id)
                s.calo_edep[det] += s.energy_deposition[i];
        }
        // ... and the step output: hits in slot order (DetectorSteps)
        if (hits_.enabled())
        {
            size_type count = 0;
            for (size_type i = 0; i < n; ++i)
            {
                if (has_step_hit(s, hits_, i))
                    write_step_hit(p, s, hits_, i, count++, iteration_);
            }
            this->print_hits(count);
        }
        ++iteration_;
        // extend-from-secondaries (end)
        {
            std::vector<char> vacant(n);
            for (size_type i = 0; i < n; ++i)
            {
                bool v;
                size_type cnt;
                locate_alive(s, i, &v, &cnt, !partitions_by_charge(p.track_order));
                vacant[i] = v;
                s.secondary_counts[i] = cnt;
            }
            size_type nv = 0;
            for (size_type i = 0; i < n; ++i)
            {
                if (vacant[i])
                    s.vacancies[nv++] = i;
            }
            c.num_vacancies = nv;
            size_type total = 0;
            for (size_type i = 0; i < n; ++i)
            {
                size_type cnt = s.secondary_counts[i];
                s.secondary_counts[i] = total;
                total += cnt;
            }
            c.num_secondaries = total;
            c.num_initializers += total;
            if (c.num_initializers > s.initializer_capacity)
                throw std::runtime_error("initializer capacity exceeded");
            c.num_alive = n - c.num_vacancies;
            for (size_type i = 0; i < n; ++i)
                process_secondaries(p, s, c, i, s.secondary_counts[i]);
        }
        StepCounts r;
        r.generated = c.num_generated;
        r.active = active;
        r.alive = c.num_alive;
        r.queued = c.num_initializers;
        return r;
    }
};

//! Physics options from the command line: --msc, --field Bx By Bz [tesla],
//! --track-order N (changes the registered actions only: the host loop's
//! results do not depend on the thread order), --reentrant-looping (a
//! reentrant boundary step keeps the looping-step count; off in the
//! reference), --rz-field FILE, --brem-combined (one combined
//! bremsstrahlung model, RunnerInput::brem_combined), --field-option NAME
//! VALUE (a FieldDriverOptions member, RunnerInput::field_options)
ParamsOptions physics_options(int argc, char** argv)
{
    ParamsOptions opts;
    for (int i = 1; i < argc; ++i)
    {
        std::string a = argv[i];
        if (a == "--msc")
            opts.msc = true;
        else if (a == "--field" && i + 3 < argc)
        {
            for (int k = 0; k < 3; ++k)
                opts.field_tesla[k] = std::strtod(argv[i + 1 + k], nullptr);
        }
        else if (a == "--track-order" && i + 1 < argc)
        {
            opts.track_order = std::stoul(argv[i + 1]);
        }
        else if (a == "--reentrant-looping")
        {
            opts.reentrant_looping = true;
        }
        else if (a == "--rz-field" && i + 1 < argc)
        {
            opts.rz_field_file = argv[i + 1];
        }
        else if (a == "--brem-combined")
        {
            opts.brem_combined = true;
        }
        else if (a == "--field-option" && i + 2 < argc)
        {
            std::string name = argv[i + 1];
            double v = std::strtod(argv[i + 2], nullptr);
            FieldOptions& o = opts.field_options;
#define GBX_FIELD_OPTION(M)                   \
    if (name == #M)                           \
        o.M = static_cast<decltype(o.M)>(v);  \
    else
            GBX_FIELD_OPTION(minimum_step)
            GBX_FIELD_OPTION(delta_chord)
            GBX_FIELD_OPTION(delta_intersection)
            GBX_FIELD_OPTION(epsilon_step)
            GBX_FIELD_OPTION(epsilon_rel_max)
            GBX_FIELD_OPTION(errcon)
            GBX_FIELD_OPTION(pgrow)
            GBX_FIELD_OPTION(pshrink)
            GBX_FIELD_OPTION(safety)
            GBX_FIELD_OPTION(max_stepping_increase)
            GBX_FIELD_OPTION(max_stepping_decrease)
            GBX_FIELD_OPTION(max_nsteps)
            GBX_FIELD_OPTION(max_substeps)
            throw std::runtime_error("unknown field option " + name);
#undef GBX_FIELD_OPTION
            i += 2;
        }
    }
    return opts;
}

std::vector<TrackInitializer> load_primaries(std::string const& path)
{
    std::ifstream in(path);
    if (!in)
        throw std::runtime_error("cannot open " + path);
    std::vector<TrackInitializer> result;
    int pdg;
    double e, x, y, z, dx, dy, dz, t;
    long ev;
    while (in >> pdg >> e >> x >> y >> z >> dx >> dy >> dz >> t >> ev)
    {
        TrackInitializer ti{};
        ti.particle_id = pdg == 11 ? 0 : (pdg == -11 ? 1 : 2);
        ti.energy = e;
        ti.pos = {x, y, z};
        ti.dir = {dx, dy, dz};
        ti.time = t;
        ti.event_id = static_cast<size_type>(ev);
        result.push_back(ti);
    }
    return result;
}

//! One interaction per input, the GB300 path's model code on tracks that its
//! own first actions prepared, as the reference harness's 'interact' mode
//! does with the reference's model actions: each input line (model label,
//! PDG, energy [MeV], position [cm], direction, element component) becomes a
//! primary of its own event; extend-from-primaries, initialize-tracks and
//! pre-step run; each track's step-limit action and element component are
//! set as physics-discrete-select would (PhysicsStepUtils.hh:253-308); the
//! named models run in action-ID order over the slots.
int interact_inputs(int argc, char** argv)
{
    if (argc < 6)
    {
        std::cerr << "usage: interact <physics> <geometry> <inputs> <seed> "
                     "[physics options]\n";
        return 2;
    }
    std::string phys = argv[2], geo = argv[3], in_path = argv[4];
    unsigned int seed = std::stoul(argv[5]);
    HostParams hp = build_params(phys, make_geometry(geo), physics_options(argc, argv));

    std::ifstream in(in_path);
    if (!in)
        throw std::runtime_error("cannot open " + in_path);
    std::vector<TrackInitializer> primaries;
    std::vector<std::string> models;
    std::vector<size_type> elcomps;
    std::string model;
    int pdg;
    double e, x, y, z, dx, dy, dz;
    size_type elcomp;
    while (in >> model >> pdg >> e >> x >> y >> z >> dx >> dy >> dz >> elcomp)
    {
        TrackInitializer ti{};
        ti.particle_id = pdg == 11 ? 0 : (pdg == -11 ? 1 : 2);
        ti.energy = e;
        ti.pos = {x, y, z};
        ti.dir = {dx, dy, dz};
        ti.time = 0;
        ti.event_id = static_cast<size_type>(primaries.size());
        primaries.push_back(ti);
        models.push_back(model);
        elcomps.push_back(elcomp);
    }
    if (primaries.empty())
        throw std::runtime_error("no inputs in " + in_path);

    size_type const n = static_cast<size_type>(primaries.size());
    PortStepper stepper(hp, n, seed, n);
    stepper.prepare(primaries);
    ParamsData const& p = stepper.params();
    StateData s = stepper.view();
    auto const& labels = stepper.action_labels();
    // The pre-step's results per input: step limit and its action, sampled
    // interaction MFP, macroscopic and per-process cross sections, range
    for (size_type i = 0; i < n; ++i)
    {
        std::printf("pre %u act=%u len=%.17g mfp=%.17g macro=%.17g range=%.17g xs=",
                    s.event_id[i],
                    s.post_step_action[i],
                    s.step_length[i],
                    double(s.interaction_mfp[i]),
                    double(s.macro_xs[i]),
                    double(s.dedx_range[i]));
        size_type const np = p.process_groups[s.particle_id[i]].num_processes;
        for (size_type k = 0; k < np; ++k)
            std::printf("%s%.17g", k ? "," : "", double(s.per_process_xs[k][i]));
        std::printf("\n");
    }
    std::vector<size_type> to_run;
    std::vector<size_type> slot_of(n);
    for (size_type i = 0; i < n; ++i)
    {
        if (s.status[i] != status_alive)
            throw std::runtime_error("track slot " + std::to_string(i)
                                     + " is not alive after pre-step");
        size_type const idx = s.event_id[i];
        auto found = std::find(labels.begin(), labels.end(), models[idx]);
        if (found == labels.end())
            throw std::runtime_error("no action '" + models[idx] + "'");
        size_type const aid = static_cast<size_type>(found - labels.begin());
        s.post_step_action[i] = aid;
        s.element[i] = elcomps[idx];
        slot_of[idx] = i;
        if (std::find(to_run.begin(), to_run.end(), aid) == to_run.end())
            to_run.push_back(aid);
    }
    std::sort(to_run.begin(), to_run.end());
    for (size_type aid : to_run)
    {
        for (size_type i = 0; i < n; ++i)
            interact(p, s, i, aid);
    }
    for (size_type idx = 0; idx < n; ++idx)
    {
        size_type const i = slot_of[idx];
        size_type const nsec = s.secondaries_count[i];
        std::printf("int %u %s st=%d act=%u mat=%u E=%.17g dir=(%.17g,%.17g,%.17g) "
                    "edep=%.17g nsec=%u rng=%u,%u,%u,%u,%u,%u\n",
                    idx,
                    models[idx].c_str(),
                    int(s.status[i]),
                    s.post_step_action[i],
                    s.material[i],
                    double(s.energy[i]),
                    s.dir[0][i], s.dir[1][i], s.dir[2][i],
                    double(s.energy_deposition[i]),
                    nsec,
                    s.rng.s[0][i], s.rng.s[1][i], s.rng.s[2][i],
                    s.rng.s[3][i], s.rng.s[4][i], s.rng.weyl[i]);
        for (size_type k = 0; k < nsec; ++k)
        {
            Secondary const& sec = s.secondaries[s.secondaries_offset[i] + k];
            std::printf("sec %u %u pdg=%d E=%.17g dir=(%.17g,%.17g,%.17g)\n",
                        idx,
                        k,
                        sec.particle_id == invalid_id ? 0 : p.particles[sec.particle_id].pdg,
                        double(sec.energy),
                        double(sec.direction[0]),
                        double(sec.direction[1]),
                        double(sec.direction[2]));
        }
    }
    return 0;
}

//! One along-step per input, as the reference harness's 'along' mode: each
//! input line (as for 'interact'; the label is not used) becomes a primary of
//! its own event; extend-from-primaries, initialize-tracks, pre-step,
//! step-gather-pre, the along-step actions and physics-discrete-select run.
int along_inputs(int argc, char** argv)
{
    if (argc < 6)
    {
        std::cerr << "usage: along <physics> <geometry> <inputs> <seed> "
                     "[physics options]\n";
        return 2;
    }
    std::string phys = argv[2], geo = argv[3], in_path = argv[4];
    unsigned int seed = std::stoul(argv[5]);
    HostParams hp = build_params(phys, make_geometry(geo), physics_options(argc, argv));

    std::ifstream in(in_path);
    if (!in)
        throw std::runtime_error("cannot open " + in_path);
    std::vector<TrackInitializer> primaries;
    std::string label;
    int pdg;
    double e, x, y, z, dx, dy, dz;
    size_type elcomp;
    while (in >> label >> pdg >> e >> x >> y >> z >> dx >> dy >> dz >> elcomp)
    {
        TrackInitializer ti{};
        ti.particle_id = pdg == 11 ? 0 : (pdg == -11 ? 1 : 2);
        ti.energy = e;
        ti.pos = {x, y, z};
        ti.dir = {dx, dy, dz};
        ti.time = 0;
        ti.event_id = static_cast<size_type>(primaries.size());
        primaries.push_back(ti);
    }
    if (primaries.empty())
        throw std::runtime_error("no inputs in " + in_path);

    size_type const n = static_cast<size_type>(primaries.size());
    PortStepper stepper(hp, n, seed, n);
    stepper.prepare(primaries);
    ParamsData const& p = stepper.params();
    StateData s = stepper.view();
    for (size_type i = 0; i < n; ++i)
        gather_pre(p, s, i);
    for (size_type i = 0; i < n; ++i)
        along_step(p, s, i);
    std::vector<size_type> along_action(s.post_step_action, s.post_step_action + n);
    for (size_type i = 0; i < n; ++i)
        discrete_select(p, s, i);
    auto const& labels = stepper.action_labels();
    size_type const rejected = static_cast<size_type>(
        std::find(labels.begin(), labels.end(), "physics-integral-rejected")
        - labels.begin());
    std::vector<size_type> slot_of(n);
    for (size_type i = 0; i < n; ++i)
        slot_of[s.event_id[i]] = i;
    for (size_type idx = 0; idx < n; ++idx)
    {
        size_type const i = slot_of[idx];
        size_type const sel = s.post_step_action[i];
        int const el = (sel != along_action[i] && sel != rejected)
                           ? static_cast<int>(s.element[i])
                           : -1;
        std::printf("along %u st=%d act=%u sel=%u el=%d len=%.17g "
                    "pos=(%.17g,%.17g,%.17g) "
                    "dir=(%.17g,%.17g,%.17g) E=%.17g edep=%.17g "
                    "rng=%u,%u,%u,%u,%u,%u\n",
                    idx,
                    int(s.status[i]),
                    along_action[i],
                    sel,
                    el,
                    s.step_length[i],
                    s.pos[0][i], s.pos[1][i], s.pos[2][i],
                    s.dir[0][i], s.dir[1][i], s.dir[2][i],
                    double(s.energy[i]),
                    double(s.energy_deposition[i]),
                    s.rng.s[0][i], s.rng.s[1][i], s.rng.s[2][i],
                    s.rng.s[3][i], s.rng.s[4][i], s.rng.weyl[i]);
    }
    return 0;
}

int run(int argc, char** argv)
{
    if (argc < 7)
    {
        std::cerr << "usage: run <physics> <geometry> <primaries> <slots> "
                     "<seed> [--steps N] [--quiet]\n";
        return 2;
    }
    std::string phys = argv[2], geo = argv[3], prim = argv[4];
    size_type slots = std::stoul(argv[5]);
    unsigned int seed = std::stoul(argv[6]);
    size_type max_steps = static_cast<size_type>(-1);
    bool quiet = false;
    bool trace = false;
    long long reseed = -1;
    size_type dump_rng = 0;
    bool hits = false;
    for (int i = 7; i < argc; ++i)
    {
        std::string a = argv[i];
        if (a == "--trace")
            trace = true;
        else if (a == "--steps")
            max_steps = std::stoul(argv[++i]);
        else if (a == "--quiet")
            quiet = true;
        else if (a == "--reseed")
            reseed = std::stoll(argv[++i]);
        else if (a == "--dump-rng")
            dump_rng = std::stoul(argv[++i]);
        else if (a == "--hits")
            hits = true;
    }
    HostParams hp = build_params(phys, make_geometry(geo), physics_options(argc, argv));
    auto primaries = load_primaries(prim);
    size_type max_event = 0;
    for (auto const& pr : primaries)
        max_event = std::max(max_event, pr.event_id);

    if (!quiet)
    {
        for (std::size_t i = 0; i < hp.action_labels.size(); ++i)
            std::printf("action %zu %s\n", i, hp.action_labels[i].c_str());
    }
    auto t0 = std::chrono::steady_clock::now();
    PortStepper step(hp, slots, seed, max_event + 1);
    if (reseed >= 0)
        step.reseed(static_cast<unsigned long long>(reseed));
    if (hits)
        step.enable_hits();
    for (size_type i = 0; i < std::min(dump_rng, slots); ++i)
    {
        auto w = step.rng_words(i);
        std::printf("rng %u %u %u %u %u %u %u\n", i, w[0], w[1], w[2], w[3], w[4], w[5]);
    }
    StepCounts counts = step(primaries);
    size_type iter = 0;
    if (trace)
        step.trace(iter);
    unsigned long long track_steps = counts.active;
    if (!quiet)
        std::printf("step %u %u %u %u %u\n",
                    iter,
                    counts.generated,
                    counts.queued,
                    counts.active,
                    counts.alive);
    while (counts && ++iter < max_steps)
    {
        counts = step();
        if (trace)
            step.trace(iter);
        track_steps += counts.active;
        if (!quiet)
            std::printf("step %u %u %u %u %u\n",
                        iter,
                        counts.generated,
                        counts.queued,
                        counts.active,
                        counts.alive);
    }
    auto t1 = std::chrono::steady_clock::now();
    std::printf("total_steps %llu iterations %u\n", track_steps, iter + 1);
    std::printf("seconds %.6f\n", std::chrono::duration<double>(t1 - t0).count());
    auto const& edep = step.edep();
    for (std::size_t i = 0; i < edep.size(); ++i)
        std::printf("edep %s %.17g\n", hp.detector_labels[i].c_str(), edep[i]);
    #ifdef GBX_CHECK_SAFE_BALL
    std::fprintf(stderr, "safe_ball uses %llu mismatches %llu\n",
                 safe_ball_uses, safe_ball_mismatches);
#endif
    return 0;
}

//! Timed CPU baseline: events distributed over threads, one stepper per
//! thread, each event transported to completion (celer-sim with
//! CELERITAS_OPENMP=event, app/celer-sim/celer-sim.cc:126-138)
int bench(int argc, char** argv)
{
    if (argc < 7)
        return 2;
    std::string phys = argv[2], geo = argv[3], prim = argv[4];
    size_type slots = std::stoul(argv[5]);
    unsigned int seed = std::stoul(argv[6]);
    unsigned int threads = 1;
    std::string tally_path;
    for (int i = 7; i < argc; ++i)
    {
        std::string a = argv[i];
        if (a == "--threads")
            threads = std::stoul(argv[++i]);
        else if (a == "--event-tallies")
            tally_path = argv[++i];
    }
    HostParams hp = build_params(phys, make_geometry(geo), physics_options(argc, argv));
    auto primaries = load_primaries(prim);
    // Group primaries by event
    std::map<size_type, std::vector<TrackInitializer>> events;
    for (auto const& p : primaries)
        events[p.event_id].push_back(p);
    std::vector<std::vector<TrackInitializer>> ev_list;
    std::vector<size_type> ev_ids;
    for (auto& kv : events)
    {
        for (auto& p : kv.second)
            p.event_id = 0;
        ev_ids.push_back(kv.first);
        ev_list.push_back(std::move(kv.second));
    }
    // Per-event deposition of every detector (the change of the stepper's
    // tally over the event), written after the timed region
    std::size_t const ndet = hp.detector_labels.size();
    std::vector<double> ev_edep(tally_path.empty() ? 0 : ev_list.size() * ndet);
    std::vector<unsigned long long> steps(threads, 0);
    std::vector<size_type> done(threads, 0);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (unsigned int t = 0; t < threads; ++t)
    {
        pool.emplace_back([&, t] {
            PortStepper step(hp, slots, seed + t, 1);
            std::vector<double> before(ndet);
            for (std::size_t e = t; e < ev_list.size(); e += threads)
            {
                if (!ev_edep.empty())
                    before = step.edep();
                StepCounts c = step(ev_list[e]);
                steps[t] += c.active;
                while (c)
                {
                    c = step();
                    steps[t] += c.active;
                }
                ++done[t];
                for (std::size_t d = 0; d < ndet && !ev_edep.empty(); ++d)
                    ev_edep[e * ndet + d] = step.edep()[d] - before[d];
            }
        });
    }
    for (auto& th : pool)
        th.join();
    auto t1 = std::chrono::steady_clock::now();
    unsigned long long total = 0;
    size_type nev = 0;
    for (unsigned int t = 0; t < threads; ++t)
    {
        total += steps[t];
        nev += done[t];
    }
    double sec = std::chrono::duration<double>(t1 - t0).count();
    std::printf("bench threads %u events %u track_steps %llu seconds %.6f\n",
                threads,
                nev,
                total,
                sec);
    if (!tally_path.empty())
    {
        std::FILE* f = std::fopen(tally_path.c_str(), "w");
        if (!f)
            throw std::runtime_error("cannot write " + tally_path);
        for (std::size_t e = 0; e < ev_list.size(); ++e)
        {
            std::fprintf(f, "%u", ev_ids[e]);
            for (std::size_t d = 0; d < ndet; ++d)
                std::fprintf(f, " %.17g", ev_edep[e * ndet + d]);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
    }
    return 0;
}

//! Random straight walks through a geometry: every query's next step and
//! safety as hexadecimal doubles, for comparing two builds of the
//! navigation (the ordered background search against a solve of every
//! surface). Usage: geo-rays <physics> <geometry> <num_walks> <seed>
int geo_rays(int argc, char** argv)
{
    if (argc < 6)
        return 2;
    HostParams hp = build_params(argv[2], make_geometry(argv[3]), ParamsOptions{});
    ParamsData const p = make_host_view(hp);
    size_type const num_walks = std::stoul(argv[4]);
    std::mt19937_64 gen(std::stoull(argv[5]));
    std::uniform_real_distribution<double> u(0.0, 1.0);
    HostState st(1, 16, 1, 16, hp.scalars.num_detectors, 0);
    StateData s = st.view();
    GeoTrackView geo(p.geo, s, 0);

    // Extent of the world box and of the cylinders
    double lo[3], hi[3];
    for (int ax = 0; ax < 3; ++ax)
    {
        lo[ax] = hp.surfaces[p.geo.world_faces[2 * ax]].value;
        hi[ax] = hp.surfaces[p.geo.world_faces[2 * ax + 1]].value;
    }
    std::vector<double> radii;
    for (auto const& sr : hp.surfaces)
    {
        if (sr.type == surf_czc)
            radii.push_back(std::sqrt(sr.value));
    }
    auto isotropic = [&] {
        double const mu = 2 * u(gen) - 1;
        double const phi = 2 * constants::pi * u(gen);
        double const st = std::sqrt(1 - mu * mu);
        return Real3{st * std::cos(phi), st * std::sin(phi), mu};
    };
    auto direction = [&] {
        double const k = u(gen);
        if (k < 0.05)
        {
            // Along an axis, or within 1e-6 of the z axis
            Real3 d{0, 0, 0};
            d[static_cast<int>(3 * u(gen)) % 3] = (u(gen) < 0.5) ? -1 : 1;
            if (u(gen) < 0.5)
                d = make_unit_vector(Real3{1e-6 * (u(gen) - 0.5), 1e-6 * (u(gen) - 0.5),
                                           (u(gen) < 0.5) ? -1.0 : 1.0});
            return d;
        }
        if (k < 0.15)
        {
            // Nearly tangent to a cylinder through the point: radial
            // component near zero
            Real3 d = isotropic();
            Real3 const r = make_unit_vector(Real3{geo.pos().x, geo.pos().y, 0});
            if (!std::isnan(r.x))
            {
                double const dr = d.x * r.x + d.y * r.y;
                d = make_unit_vector(Real3{d.x - dr * r.x * (1 - 1e-9 * u(gen)),
                                           d.y - dr * r.y * (1 - 1e-9 * u(gen)), d.z});
            }
            return d;
        }
        return isotropic();
    };
    auto max_step = [&] {
        double const k = u(gen);
        if (k < 0.3)
            return static_cast<double>(INFINITY);
        if (k < 0.35)
            return 1e10;
        return std::pow(10.0, -6 + 10 * u(gen));
    };

    size_type background = 0;
    for (size_type w = 0; w < num_walks; ++w)
    {
        Real3 pos;
        if (!radii.empty() && u(gen) < 0.7)
        {
            // Near a cylinder: a radius within 1 cm of one, or exactly on it
            double r = radii[static_cast<std::size_t>(u(gen) * radii.size()) % radii.size()];
            if (u(gen) < 0.8)
                r += 2 * u(gen) - 1;
            double const phi = 2 * constants::pi * u(gen);
            pos = {r * std::cos(phi), r * std::sin(phi),
                   lo[2] + (hi[2] - lo[2]) * u(gen)};
        }
        else
        {
            for (int ax = 0; ax < 3; ++ax)
                pos[ax] = lo[ax] + (hi[ax] - lo[ax]) * u(gen);
        }
        geo.initialize(pos, Real3{0, 0, 1});
        if (geo.failed() || geo.is_outside())
            continue;
        geo.set_dir(direction());
        for (int k = 0; k < 40; ++k)
        {
            double const step = max_step();
            Propagation const prop = geo.find_next_step(step);
            double const safety = geo.is_on_boundary() ? 0.0 : geo.find_safety();
            background += (geo.volume() == p.geo.background);
            std::printf("%u %d %u %a %d %u %a\n",
                        w,
                        k,
                        geo.volume(),
                        prop.distance,
                        prop.boundary ? 1 : 0,
                        s.next_surface[0],
                        safety);
            if (prop.boundary)
            {
                geo.move_to_boundary();
                geo.cross_boundary();
                if (geo.is_outside() || geo.failed())
                    break;
            }
            else if (std::isfinite(prop.distance))
            {
                geo.move_internal(prop.distance * u(gen));
            }
            if (u(gen) < 0.3)
                geo.set_dir(direction());
        }
    }
    std::fprintf(stderr, "background queries %u\n", background);
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 2)
    {
        std::cerr << "usage: port_stepper run ...\n";
        return 2;
    }
    try
    {
        std::string mode = argv[1];
        if (mode == "run")
            return run(argc, argv);
        if (mode == "bench")
            return bench(argc, argv);
        if (mode == "interact")
            return interact_inputs(argc, argv);
        if (mode == "along")
            return along_inputs(argc, argv);
        if (mode == "geo-rays")
            return geo_rays(argc, argv);
        if (mode == "libm" && argc >= 3)
        {
            // The FP64 elementary functions of the build (gbx/Libm.hh): one
            // hexadecimal double per input line, the result per output line
            std::string fn = argv[2];
            double x;
            while (std::scanf("%la", &x) == 1)
            {
                double y;
                if (fn == "exp")
                    y = gbx::libm::exp(x);
                else if (fn == "log")
                    y = gbx::libm::log(x);
                else if (fn == "sin")
                    y = gbx::libm::sin(x);
                else if (fn == "cos")
                    y = gbx::libm::cos(x);
                else if (fn == "tanh")
                    y = gbx::libm::tanh(x);
                else if (fn == "log1p")
                    y = gbx::libm::log1p(x);
                else if (fn == "expm1")
                    y = gbx::libm::expm1(x);
                else if (fn == "cbrt")
                    y = gbx::libm::cbrt(x);
                else
                    return 2;
                std::printf("%a\n", y);
            }
            return 0;
        }
        if (mode == "geo" && argc >= 4)
        {
            // Geometry tables built by the GB300 path's host code
            HostParams hp
                = build_params(argv[2], make_geometry(argv[3]), ParamsOptions{});
            for (std::size_t i = 0; i < hp.surfaces.size(); ++i)
                std::printf("surf %zu axis %d position %.17g\n",
                            i,
                            hp.surfaces[i].type,
                            hp.surfaces[i].value);
            for (std::size_t i = 0; i < hp.volume_labels.size(); ++i)
                std::printf("volume %zu %s\n", i, hp.volume_labels[i].c_str());
            return 0;
        }
    }
    catch (std::exception const& e)
    {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    return 2;
}
