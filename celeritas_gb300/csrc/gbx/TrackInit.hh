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

//! Initialize a vacant slot from an initializer (InitTracksExecutor)
GBX_FUNCTION void init_track(ParamsData const& p,
                             StateData const& s,
                             Counters const& counters,
                             size_type tid)
{
    TrackInitializer const& init
        = s.initializers[counters.num_initializers - tid - 1];
    size_type const slot = s.vacancies[counters.num_vacancies - tid - 1];

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
    size_type parent = invalid_id;
    if (tid < counters.num_secondaries)
    {
        parent = s.parents[s.size - tid - 1];
    }
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

//! Flag the slot as vacant or occupied and count secondaries that need a
//! new slot (LocateAliveExecutor); returns {is_vacant, num_new_secondaries}
GBX_FUNCTION void locate_alive(StateData const& s,
                               size_type slot,
                               bool* vacant,
                               size_type* count)
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
    else if (num_secondaries > 0)
    {
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
        if (!initialized && status != status_alive)
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
            if (offset <= s.size)
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
