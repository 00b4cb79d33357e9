// Track-state storage in host memory (structure of arrays), used to stage
// state to and from the device and by the host-side test driver.
#pragma once

#include <cstdint>
#include <random>
#include <vector>

#include "../gbx/Data.hh"

namespace gbx
{
//! Fill per-slot XORWOW states from a seed exactly as the reference does
//! (std::seed_seq over {seed} -> std::mt19937 -> uniform 32-bit ints; five
//! xor words then the Weyl word per slot; XorwowRngData.cc:28-63)
inline void initialize_xorwow(unsigned int seed,
                              size_type size,
                              std::vector<std::uint32_t>* words)
{
    words->resize(6 * std::size_t(size));
    std::vector<std::seed_seq::result_type> seeds{seed};
    std::seed_seq seed_seq(seeds.begin(), seeds.end());
    std::mt19937 rng(seed_seq);
    std::uniform_int_distribution<std::uint32_t> sample;
    for (size_type i = 0; i < size; ++i)
    {
        for (int w = 0; w < 6; ++w)
        {
            // word-major layout: word w of slot i at [w * size + i]
            (*words)[std::size_t(w) * size + i] = sample(rng);
        }
    }
}

//! Host-memory state with the same layout as the device state
struct HostState
{
    size_type size{0};
    std::vector<std::uint8_t> status;
    std::vector<size_type> track_id, parent_id, event_id, num_steps;
    std::vector<double> time, step_length;
    std::vector<size_type> post_step_action, along_step_action;
    std::vector<size_type> particle_id;
    std::vector<real_type> energy;
    std::vector<double> pos[3], dir[3];
    std::vector<size_type> volume, surface;
    std::vector<std::int8_t> surface_sense;
    std::vector<std::uint8_t> boundary;
    std::vector<double> next_step;
    std::vector<size_type> next_surface;
    std::vector<std::int8_t> next_sense;
    std::vector<std::uint8_t> geo_failed;
    std::vector<size_type> material;
    std::vector<real_type> interaction_mfp, dedx_range, macro_xs;
    std::vector<real_type> per_process_xs[max_processes];
    std::vector<real_type> energy_deposition;
    std::vector<size_type> secondaries_offset, secondaries_count, element;
    std::vector<std::uint8_t> msc_displaced;
    std::vector<real_type> msc_true_path, msc_geom_path, msc_alpha;
    std::vector<real_type> log_energy_key, log_energy_value;
    std::vector<size_type> init_indices;
    std::vector<real_type> msc_range_init, msc_range_factor, msc_limit_min;
    std::vector<size_type> num_looping_steps;
    std::vector<std::uint32_t> rng_words;
    std::vector<size_type> vacancies, secondary_counts, parents;
    std::vector<TrackInitializer> initializers;
    std::vector<size_type> track_counters;
    std::vector<Secondary> secondaries;
    std::vector<size_type> detector;
    std::vector<double> calo_edep;
    // Step output: pre-step points (empty unless hits are collected)
    std::vector<double> pre_time, pre_pos, pre_dir, pre_energy;
    std::vector<TrackInitializer> primaries;
    Counters counters{};

    HostState(size_type num_slots,
              size_type init_capacity,
              size_type max_events,
              size_type secondary_capacity,
              size_type num_detectors,
              unsigned int seed)
        : size(num_slots)
    {
        auto n = std::size_t(num_slots);
        status.assign(n, status_inactive);
        track_id.assign(n, invalid_id);
        parent_id.assign(n, invalid_id);
        event_id.assign(n, invalid_id);
        num_steps.assign(n, 0);
        time.assign(n, 0);
        step_length.assign(n, 0);
        post_step_action.assign(n, invalid_id);
        along_step_action.assign(n, invalid_id);
        particle_id.assign(n, invalid_id);
        energy.assign(n, 0);
        for (int i = 0; i < 3; ++i)
        {
            pos[i].assign(n, 0);
            dir[i].assign(n, 0);
        }
        volume.assign(n, invalid_id);
        surface.assign(n, invalid_id);
        surface_sense.assign(n, 0);
        boundary.assign(n, 0);
        next_step.assign(n, 0);
        next_surface.assign(n, invalid_id);
        next_sense.assign(n, 0);
        geo_failed.assign(n, 0);
        material.assign(n, invalid_id);
        interaction_mfp.assign(n, 0);
        dedx_range.assign(n, 0);
        macro_xs.assign(n, 0);
        for (auto& v : per_process_xs)
            v.assign(n, 0);
        energy_deposition.assign(n, 0);
        secondaries_offset.assign(n, 0);
        secondaries_count.assign(n, 0);
        element.assign(n, invalid_id);
        msc_displaced.assign(n, 0);
        msc_true_path.assign(n, 0);
        log_energy_key.assign(n, real_type(NAN));
        init_indices.assign(n, 0);
        log_energy_value.assign(n, 0);
        msc_geom_path.assign(n, 0);
        msc_alpha.assign(n, 0);
        msc_range_init.assign(n, 0);
        msc_range_factor.assign(n, 0);
        msc_limit_min.assign(n, 0);
        num_looping_steps.assign(n, 0);
        initialize_xorwow(seed, num_slots, &rng_words);
        // All slots start vacant, in increasing order
        vacancies.resize(n);
        for (size_type i = 0; i < num_slots; ++i)
            vacancies[i] = i;
        secondary_counts.assign(n, 0);
        parents.assign(n, invalid_id);
        initializers.resize(init_capacity);
        track_counters.assign(max_events, 0);
        secondaries.resize(secondary_capacity);
        detector.assign(n, invalid_id);
        calo_edep.assign(num_detectors, 0);
        counters.num_vacancies = num_slots;
    }

    StateData view()
    {
        StateData s{};
        s.size = size;
        s.status = status.data();
        s.track_id = track_id.data();
        s.parent_id = parent_id.data();
        s.event_id = event_id.data();
        s.num_steps = num_steps.data();
        s.time = time.data();
        s.step_length = step_length.data();
        s.post_step_action = post_step_action.data();
        s.along_step_action = along_step_action.data();
        s.particle_id = particle_id.data();
        s.energy = energy.data();
        for (int i = 0; i < 3; ++i)
        {
            s.pos[i] = pos[i].data();
            s.dir[i] = dir[i].data();
        }
        s.volume = volume.data();
        s.surface = surface.data();
        s.surface_sense = surface_sense.data();
        s.boundary = boundary.data();
        s.next_step = next_step.data();
        s.next_surface = next_surface.data();
        s.next_sense = next_sense.data();
        s.geo_failed = geo_failed.data();
        s.material = material.data();
        s.interaction_mfp = interaction_mfp.data();
        s.dedx_range = dedx_range.data();
        s.macro_xs = macro_xs.data();
        for (int i = 0; i < max_processes; ++i)
            s.per_process_xs[i] = per_process_xs[i].data();
        s.energy_deposition = energy_deposition.data();
        s.secondaries_offset = secondaries_offset.data();
        s.secondaries_count = secondaries_count.data();
        s.element = element.data();
        s.msc_displaced = msc_displaced.data();
        s.msc_true_path = msc_true_path.data();
        s.log_energy_key = log_energy_key.data();
        s.init_indices = init_indices.data();
        s.log_energy_value = log_energy_value.data();
        s.msc_geom_path = msc_geom_path.data();
        s.msc_alpha = msc_alpha.data();
        s.msc_range_init = msc_range_init.data();
        s.msc_range_factor = msc_range_factor.data();
        s.msc_limit_min = msc_limit_min.data();
        s.num_looping_steps = num_looping_steps.data();
        for (int w = 0; w < 5; ++w)
            s.rng.s[w] = rng_words.data() + std::size_t(w) * size;
        s.rng.weyl = rng_words.data() + std::size_t(5) * size;
        s.vacancies = vacancies.data();
        s.secondary_counts = secondary_counts.data();
        s.parents = parents.data();
        s.initializers = initializers.data();
        s.initializer_capacity = static_cast<size_type>(initializers.size());
        s.track_counters = track_counters.data();
        s.max_events = static_cast<size_type>(track_counters.size());
        s.secondaries = secondaries.data();
        s.secondary_capacity = static_cast<size_type>(secondaries.size());
        s.detector = detector.data();
        s.calo_edep = calo_edep.data();
        auto data_or_null = [](std::vector<double>& v) {
            return v.empty() ? nullptr : v.data();
        };
        s.pre_time = data_or_null(pre_time);
        s.pre_pos = data_or_null(pre_pos);
        s.pre_dir = data_or_null(pre_dir);
        s.pre_energy = data_or_null(pre_energy);
        s.primaries = primaries.data();
        s.primary_capacity = static_cast<size_type>(primaries.size());
        s.counters = &counters;
        return s;
    }
};

}  // namespace gbx
