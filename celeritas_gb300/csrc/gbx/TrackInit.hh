// Per-slot bodies of track creation: primaries -> initializers, initializers
// -> vacant slots, and end-of-step secondary processing.
//
// Semantics follow:
//   src/celeritas/track/detail/ProcessPrimariesExecutor.hh
//   src/celeritas/track/detail/InitTracksExecutor.hh:71-175
//   src/celeritas/track/detail/LocateAliveExecutor.hh:60-106
//   src/celeritas/track/detail/ProcessSecondariesExecutor.hh:69-183
// The order-defining rules are kept exactly: new tracks take initializers and
// vacancies from the back of their lists (index_before), the first valid
// secondary of a dead track is initialized in place, and the initializers of
// the remaining secondaries are laid out by an exclusive scan over slots.
#pragma once

#include "Actions.hh"

namespace gbx
{
//! Next track ID for an event (atomic per-event counter)
GBX_FORCEINLINE size_type make_track_id(StateData const& s, size_type event)
{
    size_type* counter = s.track_counters + event;
#if defined(__CUDA_ARCH__)
    return atomicAdd(counter, size_type(1));
#else
    return (*counter)++;
#endif
}

//! Reset per-track physics and looping state for a new track
//! (PhysicsTrackView::operator=(Initializer_t), SimTrackView init)
GBX_FORCEINLINE void reset_physics_state(StateData const& s, size_type slot)
{
    s.interaction_mfp[slot] = 0;
    s.msc_range_init[slot] = 0;
    s.msc_range_factor[slot] = 0;
    s.msc_limit_min[slot] = 0;
    s.num_looping_steps[slot] = 0;
}

//---------------------------------------------------------------------------//
// Primary generation (PrimaryGenerator, src/celeritas/phys/PrimaryGenerator.cc)
//---------------------------------------------------------------------------//
//! XORWOW stream of its own for one primary's sampling, seeded from a
//! 64-bit key like a per-track stream
struct PrimaryStream
{
    std::uint32_t s[5];
    std::uint32_t w;

    GBX_FORCEINLINE explicit PrimaryStream(std::uint64_t key)
    {
        SplitMix64 sm{key};
        std::uint64_t v = sm();
        s[0] = static_cast<std::uint32_t>(v);
        s[1] = static_cast<std::uint32_t>(v >> 32);
        v = sm();
        s[2] = static_cast<std::uint32_t>(v);
        s[3] = static_cast<std::uint32_t>(v >> 32);
        v = sm();
        s[4] = static_cast<std::uint32_t>(v);
        w = static_cast<std::uint32_t>(v >> 32);
        if ((s[0] | s[1] | s[2] | s[3] | s[4]) == 0)
            s[0] = 1;
    }
    GBX_FORCEINLINE std::uint32_t operator()()
    {
        std::uint32_t const t = (s[0] ^ (s[0] >> 2u));
        s[0] = s[1];
        s[1] = s[2];
        s[2] = s[3];
        s[3] = s[4];
        s[4] = (s[4] ^ (s[4] << 4u)) ^ (t ^ (t << 1u));
        w += 362437u;
        return w + s[4];
    }
};

//! Key of the per-track stream of primary 'index' of an event: the
//! stepper seed, the event and the primary's index among its event's
//! primaries (the same key as a primary inserted from the host)
GBX_FORCEINLINE std::uint64_t
primary_stream_key(unsigned int seed, size_type event, size_type index)
{
    SplitMix64 sm{(std::uint64_t(seed) << 32) | event};
    SplitMix64 sm2{sm() + 0x9e3779b97f4a7c15ull * (std::uint64_t(index) + 1)};
    return sm2();
}

//! Sample primary 'tid' of a generator launch into the staged primaries
//! (PrimaryGenerator::operator(): particle cycled by index within the
//! event, energy, then position, then direction, time zero). Each primary
//! samples from its own stream, keyed by the generator seed, the event and
//! the index, so any subset of primaries can be generated in parallel.
GBX_FUNCTION void generate_primary(PrimaryGeneratorData const& g,
                                   TrackInitializer* primaries,
                                   size_type tid)
{
    size_type const index = tid % g.primaries_per_event;
    size_type const event = g.first_event + tid / g.primaries_per_event;
    PrimaryStream rng(primary_stream_key(g.seed, event, index) ^ 0x6a09e667f3bcc909ull);
    TrackInitializer& p = primaries[tid];
    p.track_id = invalid_id;
    p.parent_id = invalid_id;
    p.event_id = event;
    p.time = 0;
    p.particle_id = g.particle_ids[index % g.num_particles];
    p.energy = real_type(g.energy);
    if (g.position_dist == dist_box)
    {
        // UniformBoxDistribution: each coordinate uniform in [lo, hi)
        for (int i = 0; i < 3; ++i)
        {
            double const u = generate_canonical<double>(rng);
            p.pos[i] = g.position[i] + u * (g.position[3 + i] - g.position[i]);
        }
    }
    else
    {
        p.pos = {g.position[0], g.position[1], g.position[2]};
    }
    if (g.direction_dist == dist_isotropic)
    {
        // IsotropicDistribution: cos(theta) uniform in [-1, 1), phi in
        // [0, 2 pi)
        double const mu = 2 * generate_canonical<double>(rng) - 1;
        double const phi = 2 * constants::pi * generate_canonical<double>(rng);
        double const sintheta = std::sqrt(1 - mu * mu);
        p.dir = {sintheta * libm::cos(phi), sintheta * libm::sin(phi), mu};
    }
    else
    {
        p.dir = {g.direction[0], g.direction[1], g.direction[2]};
    }
    p.rng_key = primary_stream_key(g.stepper_seed, event, index);
}

//! Copy primary 'tid' into the initializer list (ProcessPrimariesExecutor)
GBX_FUNCTION void process_primary(StateData const& s,
                                  size_type num_initializers,
                                  size_type num_primaries,
                                  size_type tid)
{
    TrackInitializer const& primary = s.primaries[tid];
    TrackInitializer& ti = s.initializers[num_initializers - num_primaries + tid];
    ti = primary;
    ti.track_id = make_track_id(s, primary.event_id);
    ti.parent_id = invalid_id;
}

//! Initialize vacant slot 'slot' from an initializer, copying the geometry
//! state of slot 'parent' if valid (InitTracksExecutor)
GBX_FUNCTION void init_track_from(ParamsData const& p,
                                  StateData const& s,
                                  TrackInitializer const& init,
                                  size_type slot,
                                  size_type parent)
{
    // Sim state
    s.track_id[slot] = init.track_id;
    s.parent_id[slot] = init.parent_id;
    s.event_id[slot] = init.event_id;
    s.num_steps[slot] = 0;
    s.time[slot] = init.time;
    s.status[slot] = status_initializing;
    s.step_length[slot] = 0;
    s.post_step_action[slot] = invalid_id;
    s.along_step_action[slot] = invalid_id;
    // Particle state
    s.particle_id[slot] = init.particle_id;
    s.energy[slot] = init.energy;

    // Geometry: copy the parent's state or locate from scratch
    GeoTrackView geo(p.geo, s, slot);
    if (parent != invalid_id)
    {
        geo.copy_from(parent, init.dir);
    }
    else
    {
        geo.initialize(init.pos, init.dir);
        if (geo.failed() || geo.is_outside())
        {
            apply_errored(p, s, slot);
            return;
        }
    }
    size_type matid = p.geo.volume_material[geo.volume()];
    if (matid == invalid_id)
    {
        apply_errored(p, s, slot);
        return;
    }
    s.material[slot] = matid;
    // Physics state reset
    reset_physics_state(s, slot);
    if (p.rng_per_track)
    {
        seed_xorwow(s.rng, slot, init.rng_key);
    }
}

//! Initialize vacant slot 'slot' from initializer 'tid' counted from the
//! back of the list; the first num_secondaries new tracks may have a parent
//! slot to copy the geometry from
GBX_FUNCTION void init_track_at(ParamsData const& p,
                                StateData const& s,
                                Counters const& counters,
                                size_type tid,
                                size_type slot)
{
    size_type parent = invalid_id;
    if (tid < counters.num_secondaries)
    {
        parent = s.parents[s.size - tid - 1];
    }
    init_track_from(
        p, s, s.initializers[counters.num_initializers - tid - 1], slot, parent);
}

//! Initialize a vacant slot from an initializer: new track 'tid' takes the
//! tid-th initializer and vacancy from the back of their lists
//! (InitTracksExecutor)
GBX_FUNCTION void init_track(ParamsData const& p,
                             StateData const& s,
                             Counters const& counters,
                             size_type tid)
{
    init_track_at(
        p, s, counters, tid, s.vacancies[counters.num_vacancies - tid - 1]);
}

//! Whether an initializer is neutral (IsNeutral, src/celeritas/track/
//! detail/Utils.hh:34-46)
GBX_FORCEINLINE bool is_neutral(ParamsData const& p, TrackInitializer const& init)
{
    return p.particles[init.particle_id].charge == 0;
}

//! Initialize new track 'tid' with the charge partition (TrackOrder
//! init_charge; InitTracksExecutor.hh:71-108): s.init_indices lists the
//! last num_new initializers neutral ones first, and thread 'tid' takes
//! entry num_new - tid - 1 of it. A neutral track takes the vacancy at the
//! same position from the front of the list's first num_new entries, a
//! charged one the tid-th from the back of the whole list, so that charged
//! and neutral tracks fill the two ends of the vacant slots. The parent
//! slot, for the first num_secondaries threads, is at the same partitioned
//! position of the parent list.
GBX_FUNCTION void init_track_charge_partitioned(ParamsData const& p,
                                                StateData const& s,
                                                Counters const& counters,
                                                size_type num_new,
                                                size_type tid)
{
    size_type const j = s.init_indices[num_new - tid - 1];
    TrackInitializer const& init
        = s.initializers[j + counters.num_initializers - num_new];
    size_type const slot = is_neutral(p, init)
                               ? s.vacancies[num_new - tid - 1]
                               : s.vacancies[counters.num_vacancies - tid - 1];
    size_type parent = invalid_id;
    if (tid < counters.num_secondaries)
    {
        parent = s.parents[j + s.size - num_new];
    }
    init_track_from(p, s, init, slot, parent);
}

//! Flag the slot as vacant or occupied and count secondaries that need a
//! new slot (LocateAliveExecutor); returns {is_vacant, num_new_secondaries}
GBX_FUNCTION void locate_alive(StateData const& s,
                               size_type slot,
                               bool* vacant,
                               size_type* count,
                               bool in_place = true)
{
    size_type num_secondaries = 0;
    std::uint8_t const status = s.status[slot];
    if (status != status_inactive)
    {
        Secondary const* sec = s.secondaries + s.secondaries_offset[slot];
        size_type n = s.secondaries_count[slot];
        for (size_type i = 0; i < n; ++i)
        {
            if (sec[i].particle_id != invalid_id)
                ++num_secondaries;
        }
    }
    if (status == status_alive)
    {
        *vacant = false;
    }
    else if (num_secondaries > 0 && in_place)
    {
        // The first secondary will take the dead track's slot (not with
        // the charge partition, which initializes every secondary from the
        // queue)
        --num_secondaries;
        *vacant = false;
    }
    else
    {
        *vacant = true;
    }
    *count = num_secondaries;
}

//! Create initializers for a slot's secondaries (ProcessSecondariesExecutor).
//! 'prefix' is the exclusive scan of secondary counts at this slot.
GBX_FUNCTION void process_secondaries(ParamsData const& p,
                                      StateData const& s,
                                      Counters const& counters,
                                      size_type slot,
                                      size_type prefix)
{
    std::uint8_t status = s.status[slot];
    if (status == status_inactive)
        return;
    size_type offset = counters.num_secondaries - prefix;
    bool initialized = false;
    size_type const parent_track = s.track_id[slot];
    Secondary const* sec = s.secondaries + s.secondaries_offset[slot];
    size_type const n = s.secondaries_count[slot];
    // Per-track streams: each secondary's seed is drawn from its parent's
    // stream, in secondary order, before the slot is reused
    std::uint64_t in_place_key = 0;
    for (size_type i = 0; i < n; ++i)
    {
        Secondary const& secondary = sec[i];
        if (secondary.particle_id == invalid_id)
            continue;
        TrackInitializer ti;
        ti.rng_key = 0;
        if (p.rng_per_track)
        {
            XorwowEngine parent_rng(s.rng, slot);
            std::uint64_t const lo = parent_rng();
            std::uint64_t const hi = parent_rng();
            ti.rng_key = (hi << 32) | lo;
        }
        ti.track_id = make_track_id(s, s.event_id[slot]);
        ti.parent_id = parent_track;
        ti.event_id = s.event_id[slot];
        ti.time = s.time[slot];
        ti.pos = {s.pos[0][slot], s.pos[1][slot], s.pos[2][slot]};
        ti.dir = to_geo_dir(secondary.direction);
        ti.particle_id = secondary.particle_id;
        ti.energy = secondary.energy;
        if (!initialized && status != status_alive
            && !partitions_by_charge(p.track_order))
        {
            // Reuse this slot for the first secondary
            s.track_id[slot] = ti.track_id;
            s.parent_id[slot] = ti.parent_id;
            s.event_id[slot] = ti.event_id;
            s.num_steps[slot] = 0;
            s.time[slot] = ti.time;
            s.status[slot] = status_initializing;
            s.step_length[slot] = 0;
            s.post_step_action[slot] = invalid_id;
            s.along_step_action[slot] = invalid_id;
            GeoTrackView geo(p.geo, s, slot);
            geo.copy_from(slot, ti.dir);
            s.particle_id[slot] = ti.particle_id;
            s.energy[slot] = ti.energy;
            reset_physics_state(s, slot);
            in_place_key = ti.rng_key;
            initialized = true;
            status = status_initializing;
        }
        else
        {
            s.initializers[counters.num_initializers - offset] = ti;
            // With the charge partition a secondary copies the geometry of
            // a parent that is still alive only (its slot is not reused)
            if (offset <= s.size
                && (!partitions_by_charge(p.track_order) || status == status_alive))
            {
                s.parents[s.size - offset] = slot;
            }
            --offset;
        }
    }
    if (initialized && p.rng_per_track)
    {
        seed_xorwow(s.rng, slot, in_place_key);
    }
    if (!initialized && s.status[slot] == status_killed)
    {
        s.status[slot] = status_inactive;
    }
}

}  // namespace gbx
