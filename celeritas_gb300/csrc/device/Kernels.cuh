// Kernel declarations for the GB300 stepping loop.
#pragma once

#include <cuda_runtime.h>

#include "../gbx/Data.hh"

namespace gbx
{
//! Per-step counter record kept on the device (StepperResult)
struct StepRecord
{
    size_type generated;
    size_type queued;
    size_type active;
    size_type alive;
};

//! Scratch for the end-of-step compaction: per-block totals and offsets
struct ScanScratch
{
    size_type* block_vacant;  //!< [num_blocks]
    size_type* block_count;  //!< [num_blocks]
    std::uint8_t* vacant;  //!< [num_slots]
    size_type* count;  //!< [num_slots]
    size_type num_blocks;
};

//! Scratch of the action sort: per-block bin counts, bin-major
//! ([bin][block]), for blocks of sort_block_size slots
struct SortScratch
{
    size_type* block_hist;  //!< [num_bins * num_blocks]
    //! num_actions + num_materials + 1 (last: invalid action)
    size_type num_bins;
    size_type num_blocks;
    size_type num_actions;
    size_type num_materials;
    //! TrackOrder of the parameters (the start sort's key: status or
    //! particle type)
    unsigned int track_order;
    //! Along-step sort by material within up to two actions (ascending IDs,
    //! invalid_id where unused): such an action's tracks take num_materials
    //! bins by their material, and the bins of later actions shift by
    //! num_materials - 1
    size_type material_actions[2];
};

//! Bin of a track of along-step action 'a' (a valid action ID) and material
//! 'mat' in the along-step sort; mat = 0 gives the action's first bin
__host__ __device__ inline size_type
along_bin(SortScratch const& srt, size_type a, size_type mat)
{
    size_type shift = 0;
    for (int i = 0; i < 2; ++i)
    {
        size_type const m = srt.material_actions[i];
        if (m == invalid_id)
            break;
        if (a == m)
            return a + shift + mat;
        if (a > m)
            shift += srt.num_materials - 1;
    }
    return a + shift;
}

//! Bins [first, end) of an action in the along-step sort
inline void along_bins(SortScratch const& srt, size_type action, size_type* first, size_type* end)
{
    bool const by_material = action == srt.material_actions[0]
                             || action == srt.material_actions[1];
    *first = along_bin(srt, action, 0);
    *end = *first + (by_material ? srt.num_materials : 1);
}

//! Which action a sort orders tracks by
enum class SortKey
{
    along_step,  //!< along_step_action (reindex_along_step_action)
    step_limit,  //!< post_step_action (reindex_step_limit_action)
    start,  //!< status or particle type (reindex_status, _particle_type)
};

//! Error flags written by device code
enum ErrorFlag : size_type
{
    error_initializer_overflow = 1u << 0,
    error_primary_overflow = 1u << 1,
    //! A step's hits did not fit in the step output: that step's and later
    //! steps' hits are dropped until the host reads the output
    error_hit_overflow = 1u << 2,
};

constexpr int block_size = 256;
constexpr int sort_block_size = 1024;

struct LaunchContext
{
    ParamsData params;
    StateData state;
    ScanScratch scratch;
    SortScratch sort;
    //! Grid of the persistent charged along-step kernel (0: not used) and
    //! its device work counter
    int persistent_blocks;
    size_type* work_counter;
    //! Tuning: threads per block of the charged along-step kernels (at most
    //! block_size) and whether the action sorts run this step
    int along_block_size;
    //! Grid of the short sorted-range kernels (grid-stride loops): a few
    //! blocks per SM, at most one block per block_size slots
    unsigned int range_blocks;
    bool sort_enabled;
    //! Tuning: new charged tracks take the lowest vacant slots and neutral
    //! ones the highest (per-track random streams only), so that each
    //! along-step kernel's sorted range covers mostly contiguous slots
    bool partition_slots;
    StepRecord* log;  //!< Step log (ring buffer)
    size_type log_capacity;
    size_type* step_index;  //!< Device-resident step counter
    //! Step output (disabled: zero capacity) and its per-block hit counts
    StepHitsRef hits;
    size_type* hit_block_offsets;  //!< [num_blocks_for(size)]
};

// Individual action launchers (one thread per track slot)
void launch_process_primaries(LaunchContext const& ctx,
                              size_type num_primaries,
                              cudaStream_t stream);
void launch_initialize_tracks(LaunchContext const& ctx, cudaStream_t stream);
//! Sample num_events x primaries_per_event primaries into the staged
//! primaries (PrimaryGenerator on the device)
void launch_generate_primaries(LaunchContext const& ctx,
                               PrimaryGeneratorData const& gen,
                               cudaStream_t stream);
void launch_pre_step(LaunchContext const& ctx, cudaStream_t stream);
//! Along-step for tracks whose along-step action matches (all if invalid)
void launch_along_step(LaunchContext const& ctx,
                       size_type action,
                       cudaStream_t stream);
void launch_discrete_select(LaunchContext const& ctx, cudaStream_t stream);
void launch_interact(LaunchContext const& ctx,
                     size_type action,
                     cudaStream_t stream);
void launch_boundary(LaunchContext const& ctx, cudaStream_t stream);
void launch_tracking_cut(LaunchContext const& ctx, cudaStream_t stream);
//! SimpleCalo tally and, when enabled, the step output (step-gather-post)
void launch_calo_tally(LaunchContext const& ctx, cudaStream_t stream);
void launch_extend_from_secondaries(LaunchContext const& ctx,
                                    cudaStream_t stream);
void launch_kill_active(LaunchContext const& ctx, cudaStream_t stream);
//! Reseed every slot's XORWOW state for an event: slot i gets the state of
//! 'seed' advanced event * size + i subsequences (reseed_rng)
void launch_reseed(LaunchContext const& ctx,
                   unsigned int seed,
                   unsigned long long event_id,
                   cudaStream_t stream);
//! Resident blocks of the persistent charged along-step kernel on the
//! current device (SMs x blocks per SM at full occupancy), 0 on failure
int persistent_along_blocks(int threads_per_block);
//! Count live tracks (slots and queued initializers) of events [0, n) into
//! state.event_live
void launch_count_event_live(LaunchContext const& ctx,
                             size_type num_events,
                             cudaStream_t stream);
//! Stable counting sort of the track slots by action (SortTracksAction):
//! fills state.track_slots and state.action_offsets
void launch_sort_tracks(LaunchContext const& ctx, SortKey key, cudaStream_t stream);

//! Largest state that the library-owned extend-from-secondaries scratch fits
constexpr size_type static_scratch_max_slots = 131072;
//! Extend-from-secondaries with its scratch in a static device array of the
//! library (no allocation; throws if the state has too many slots). The
//! first call on a device looks up the array's address on that device.
//! Device address of the static scratch on the current device, looked up
//! (cudaGetSymbolAddress) on the first call per device and cached
unsigned char* static_scratch_for_current_device();
void launch_extend_from_secondaries_static(LaunchContext const& ctx,
                                           cudaStream_t stream);

}  // namespace gbx
