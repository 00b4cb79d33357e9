// CUDA kernels of the GB300 stepping loop.
//
// Each action kernel runs one thread per track slot and calls the same
// per-slot function as the reference's action executor (see gbx/Actions.hh
// and gbx/TrackInit.hh). Counters stay on the device: the number of new
// tracks, vacancies, secondaries and initializers are read and updated by
// kernels, so a whole step is a fixed sequence of launches that a CUDA graph
// can capture (the reference copies counters to the host several times per
// step, src/celeritas/track/detail/TrackInitAlgorithms.cu:34-78).
//
// End-of-step bookkeeping (src/celeritas/track/ExtendFromSecondariesAction.cc)
// is three kernels: per-slot vacancy flags and secondary counts with
// per-block totals (warp ballot/popc and shuffle scans), one block scanning
// the block totals and updating the counters, and a scatter that writes the
// stably compacted vacancy list and processes each slot's secondaries at its
// exclusive-scan offset.
#include "Kernels.cuh"

#include <mutex>
#include <stdexcept>
#include <string>

#include "../gbx/TrackInit.hh"

namespace gbx
{
namespace
{
__device__ __forceinline__ size_type thread_slot()
{
    return blockIdx.x * blockDim.x + threadIdx.x;
}

inline unsigned int num_blocks_for(size_type n)
{
    return static_cast<unsigned int>((n + block_size - 1) / block_size);
}

//---------------------------------------------------------------------------//
// Block-wide exclusive scan of one 32-bit value per thread (256 threads)
//---------------------------------------------------------------------------//
struct BlockScanStorage
{
    size_type warp_sums[block_size / 32];
    size_type total;
};

__device__ __forceinline__ size_type block_exclusive_scan(size_type value,
                                                          BlockScanStorage& tmp,
                                                          size_type* total)
{
    int const lane = threadIdx.x & 31;
    int const warp = threadIdx.x >> 5;
    // Inclusive warp scan
    size_type incl = value;
#pragma unroll
    for (int offset = 1; offset < 32; offset <<= 1)
    {
        size_type n = __shfl_up_sync(0xffffffffu, incl, offset);
        if (lane >= offset)
            incl += n;
    }
    if (lane == 31)
        tmp.warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        constexpr int nwarps = block_size / 32;
        size_type w = (lane < nwarps) ? tmp.warp_sums[lane] : 0;
        size_type wincl = w;
#pragma unroll
        for (int offset = 1; offset < nwarps; offset <<= 1)
        {
            size_type n = __shfl_up_sync(0xffffffffu, wincl, offset);
            if (lane >= offset)
                wincl += n;
        }
        if (lane < nwarps)
            tmp.warp_sums[lane] = wincl - w;  // exclusive warp offsets
        if (lane == nwarps - 1)
            tmp.total = wincl;
    }
    __syncthreads();
    size_type result = tmp.warp_sums[warp] + incl - value;
    *total = tmp.total;
    __syncthreads();
    return result;
}

//---------------------------------------------------------------------------//
// Primaries and track initialization
//---------------------------------------------------------------------------//
__global__ void begin_primaries_kernel(StateData s, size_type num_primaries)
{
    Counters& c = *s.counters;
    if (num_primaries > s.initializer_capacity - c.num_initializers)
    {
        // The queue would overflow: drop the primaries, keep every queued
        // initializer valid, and let the host report the overflow
        c.error_flags |= error_initializer_overflow;
        c.num_generated = 0;
        c.num_pending_primaries = 0;
        return;
    }
    c.num_initializers += num_primaries;
    c.num_generated = num_primaries;
    c.num_pending_primaries = num_primaries;
}

__global__ void process_primaries_kernel(StateData s, size_type num_primaries)
{
    size_type tid = thread_slot();
    Counters const& c = *s.counters;
    if (tid < num_primaries && !(c.error_flags & error_initializer_overflow))
    {
        process_primary(s, c.num_initializers, num_primaries, tid);
    }
    // Primaries have no parents: clear the parent list
    for (size_type i = tid; i < s.size; i += gridDim.x * blockDim.x)
    {
        s.parents[i] = invalid_id;
    }
}

__global__ __launch_bounds__(block_size) void generate_primaries_kernel(
    PrimaryGeneratorData g, StateData s, size_type num)
{
    size_type const tid = thread_slot();
    if (tid < num)
        generate_primary(g, s.primaries, tid);
}

__global__ __launch_bounds__(block_size) void initialize_tracks_kernel(
    ParamsData p, StateData s)
{
    // Grid-stride over the new tracks, whose number is on the device
    Counters const c = *s.counters;
    size_type const num_new = min_of(c.num_vacancies, c.num_initializers);
    size_type const stride = gridDim.x * blockDim.x;
    for (size_type tid = thread_slot(); tid < num_new; tid += stride)
    {
        init_track(p, s, c, tid);
    }
}

//! Track initialization with partitioned slots: the same initializers as
//! initialize_tracks_kernel, but a charged track takes the next vacancy from
//! the front of the (ascending) list and a neutral one the next from the
//! back. The front and back runs together cover num_new distinct vacancies;
//! the vacancies left between them are not read again before the end of the
//! step rebuilds the list. Which slot a track gets depends on the order in
//! which warps claim them, which is why this needs per-track random streams.
__global__ __launch_bounds__(block_size) void initialize_tracks_partitioned_kernel(
    ParamsData p, StateData s)
{
    size_type tid = thread_slot();
    Counters const c = *s.counters;
    size_type num_new = min_of(c.num_vacancies, c.num_initializers);
    if (blockIdx.x * blockDim.x >= num_new)
        return;
    bool const valid = tid < num_new;
    bool charged = false;
    if (valid)
    {
        TrackInitializer const& init = s.initializers[c.num_initializers - tid - 1];
        charged = p.particles[init.particle_id].charge != 0;
    }
    // One atomic per warp and side: ranks within the warp by ballot
    unsigned int const lane = threadIdx.x & 31u;
    unsigned int const lt = (1u << lane) - 1u;
    unsigned int const front = __ballot_sync(0xffffffffu, valid && charged);
    unsigned int const back = __ballot_sync(0xffffffffu, valid && !charged);
    size_type front_base = 0;
    size_type back_base = 0;
    if (lane == 0)
    {
        if (front)
            front_base = atomicAdd(&s.counters->num_taken_front, __popc(front));
        if (back)
            back_base = atomicAdd(&s.counters->num_taken_back, __popc(back));
    }
    front_base = __shfl_sync(0xffffffffu, front_base, 0);
    back_base = __shfl_sync(0xffffffffu, back_base, 0);
    if (!valid)
        return;
    size_type const slot
        = charged ? s.vacancies[front_base + __popc(front & lt)]
                  : s.vacancies[c.num_vacancies - 1 - back_base - __popc(back & lt)];
    init_track_at(p, s, c, tid, slot);
}

//---------------------------------------------------------------------------//
// Charge partition of new tracks (TrackOrder init_charge): a stable
// partition of the last num_new initializers, neutral ones first
// (partition_initializers, src/celeritas/track/detail/
// TrackInitAlgorithms.cc:75-95), as a per-block count, a scan of the block
// counts and a scatter that ranks each initializer within its group. The
// end-of-step scan scratch is free at the start of the step: block_vacant
// holds the neutral count of each block, count[0] the total.
//---------------------------------------------------------------------------//
__device__ __forceinline__ bool new_track_is_neutral(ParamsData const& p,
                                                     StateData const& s,
                                                     Counters const& c,
                                                     size_type num_new,
                                                     size_type i)
{
    return i < num_new
           && is_neutral(p, s.initializers[c.num_initializers - num_new + i]);
}

__global__ __launch_bounds__(block_size) void charge_partition_count_kernel(
    ParamsData p, StateData s, ScanScratch scr)
{
    Counters const c = *s.counters;
    size_type const num_new = min_of(c.num_vacancies, c.num_initializers);
    bool const neutral = new_track_is_neutral(p, s, c, num_new, thread_slot());
    int const n = __syncthreads_count(neutral);
    if (threadIdx.x == 0)
        scr.block_vacant[blockIdx.x] = static_cast<size_type>(n);
}

__global__ __launch_bounds__(1024) void charge_partition_scan_kernel(ScanScratch scr)
{
    // Exclusive scan of the per-block neutral counts by one block
    __shared__ size_type sh[1024];
    __shared__ size_type carry;
    if (threadIdx.x == 0)
        carry = 0;
    __syncthreads();
    for (size_type base = 0; base < scr.num_blocks; base += 1024)
    {
        size_type const i = base + threadIdx.x;
        size_type const v = i < scr.num_blocks ? scr.block_vacant[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1)
        {
            size_type const a = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += a;
            __syncthreads();
        }
        if (i < scr.num_blocks)
            scr.block_vacant[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023)
            carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        scr.count[0] = carry;
}

__global__ __launch_bounds__(block_size) void charge_partition_scatter_kernel(
    ParamsData p, StateData s, ScanScratch scr)
{
    __shared__ size_type warp_neutral[block_size / 32];
    Counters const c = *s.counters;
    size_type const num_new = min_of(c.num_vacancies, c.num_initializers);
    size_type const i = thread_slot();
    bool const neutral = new_track_is_neutral(p, s, c, num_new, i);
    unsigned int const lane = threadIdx.x & 31u;
    unsigned int const warp = threadIdx.x >> 5;
    unsigned int const ballot = __ballot_sync(0xffffffffu, neutral);
    if (lane == 0)
        warp_neutral[warp] = __popc(ballot);
    __syncthreads();
    size_type before = scr.block_vacant[blockIdx.x] + __popc(ballot & ((1u << lane) - 1u));
    for (unsigned int w = 0; w < warp; ++w)
        before += warp_neutral[w];
    if (i < num_new)
    {
        size_type const pos = neutral ? before : scr.count[0] + (i - before);
        s.init_indices[pos] = i;
    }
}

__global__ __launch_bounds__(block_size) void initialize_tracks_charge_kernel(
    ParamsData p, StateData s)
{
    Counters const c = *s.counters;
    size_type const num_new = min_of(c.num_vacancies, c.num_initializers);
    size_type const stride = gridDim.x * blockDim.x;
    for (size_type tid = thread_slot(); tid < num_new; tid += stride)
        init_track_charge_partitioned(p, s, c, num_new, tid);
}

//! Clear stale parent slots after the charge-partitioned initialization
__global__ __launch_bounds__(block_size) void clear_parents_kernel(StateData s)
{
    size_type const stride = gridDim.x * blockDim.x;
    for (size_type i = thread_slot(); i < s.size; i += stride)
        s.parents[i] = invalid_id;
}

__global__ void finish_initialize_kernel(StateData s,
                                         StepRecord* log,
                                         size_type log_capacity,
                                         size_type* step_index)
{
    Counters& c = *s.counters;
    size_type num_new = min_of(c.num_vacancies, c.num_initializers);
    c.num_initializers -= num_new;
    c.num_vacancies -= num_new;
    c.num_taken_front = 0;
    c.num_taken_back = 0;
    c.num_active = s.size - c.num_vacancies;
    // pre-step clears the secondary stack
    c.secondary_stack_size = 0;
    StepRecord& r = log[*step_index % log_capacity];
    r.generated = c.num_generated;
    r.active = c.num_active;
    c.num_generated = 0;
}

//---------------------------------------------------------------------------//
// Physics actions
//---------------------------------------------------------------------------//
__global__ __launch_bounds__(block_size) void pre_step_kernel(ParamsData p,
                                                              StateData s)
{
    size_type slot = thread_slot();
    if (slot < s.size)
    {
        pre_step(p, s, slot);
        gather_pre(p, s, slot);
    }
}

__global__ __launch_bounds__(block_size) void discrete_select_kernel(
    ParamsData p, StateData s)
{
    size_type slot = thread_slot();
    if (slot < s.size)
    {
        discrete_select(p, s, slot);
    }
}

//! Add each lane's value to bins[key] with one atomic per distinct key of
//! the warp: lanes with equal keys are grouped (__match_any_sync), each
//! group's values are summed in lane order, and the group's lowest lane adds
//! the sum. Lanes with an invalid key take part in the exchange only. Every
//! lane of the warp must call this.
__device__ __forceinline__ void warp_tally(double* bins, size_type key, double value)
{
    unsigned int const active = __activemask();
    if (__ballot_sync(active, key != invalid_id) == 0)
        return;
    unsigned int const lane = threadIdx.x & 31u;
    unsigned int const group = __match_any_sync(active, key);
    double sum = 0;
    for (unsigned int k = 0; k < 32; ++k)
    {
        if (!((active >> k) & 1u))
            continue;
        double const v = __shfl_sync(active, value, k);
        if ((group >> k) & 1u)
            sum += v;
    }
    if (key != invalid_id && lane == static_cast<unsigned int>(__ffs(group) - 1))
        atomicAdd(bins + key, sum);
}

//! SimpleCalo tally (SimpleCaloExecutor, src/celeritas/user/detail/
//! SimpleCaloExecutor.hh:48-67): the step's deposition of every track in a
//! detector volume. A zero deposit leaves the sums unchanged and is skipped,
//! as the reference's step filter does; the rest is aggregated per warp.
__global__ __launch_bounds__(block_size) void calo_kernel(ParamsData p, StateData s)
{
    size_type const slot = thread_slot();
    size_type det = invalid_id;
    size_type event = invalid_id;
    double edep = 0;
    if (slot < s.size && s.status[slot] != status_inactive)
    {
        edep = s.energy_deposition[slot];
        if (edep != 0)
        {
            det = s.detector[slot];
            if (p.event_tallies && det != invalid_id)
                event = s.event_id[slot];
        }
    }
    warp_tally(s.calo_edep, det, edep);
    if (p.event_tallies)
    {
        warp_tally(s.event_edep, event, edep);
        warp_tally(s.event_det_edep,
                   event == invalid_id ? invalid_id : event * p.num_detectors + det,
                   edep);
    }
}

//---------------------------------------------------------------------------//
// Step output: each step's hits appended in slot order (DetectorSteps)
//---------------------------------------------------------------------------//
//! Hits of each block of slots
__global__ __launch_bounds__(block_size) void hits_count_kernel(StateData s,
                                                                StepHitsRef h,
                                                                size_type* block_hits)
{
    size_type const slot = thread_slot();
    bool const hit = slot < s.size && has_step_hit(s, h, slot);
    int const count = __syncthreads_count(hit);
    if (threadIdx.x == 0)
        block_hits[blockIdx.x] = static_cast<size_type>(count);
}

//! Record offsets of the blocks: the hits already held plus an exclusive
//! scan of the block counts, by one block of 1024 threads. A step whose hits
//! do not fit sets the overflow flag and records none.
__global__ __launch_bounds__(1024) void hits_scan_kernel(StateData s,
                                                         size_type* block_hits,
                                                         size_type num_blocks,
                                                         size_type capacity)
{
    __shared__ size_type sh[1024];
    __shared__ size_type carry;
    Counters& c = *s.counters;
    if (threadIdx.x == 0)
        carry = c.num_hits;
    __syncthreads();
    for (size_type base = 0; base < num_blocks; base += 1024)
    {
        size_type const i = base + threadIdx.x;
        size_type const v = i < num_blocks ? block_hits[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1)
        {
            size_type const a = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += a;
            __syncthreads();
        }
        if (i < num_blocks)
            block_hits[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023)
            carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        if (carry > capacity)
            c.error_flags |= error_hit_overflow;
        else if (!(c.error_flags & error_hit_overflow))
            c.num_hits = carry;
    }
}

//! Write each hit at its block offset plus its rank among the block's hits
__global__ __launch_bounds__(block_size) void hits_scatter_kernel(
    ParamsData p,
    StateData s,
    StepHitsRef h,
    size_type const* block_offsets,
    size_type const* step_index)
{
    __shared__ size_type warp_hits[block_size / 32];
    size_type const slot = thread_slot();
    bool const hit = slot < s.size && has_step_hit(s, h, slot);
    unsigned int const ballot = __ballot_sync(0xffffffffu, hit);
    int const lane = threadIdx.x & 31;
    int const warp = threadIdx.x >> 5;
    if (lane == 0)
        warp_hits[warp] = __popc(ballot);
    __syncthreads();
    if (!hit || (s.counters->error_flags & error_hit_overflow))
        return;
    size_type index = block_offsets[blockIdx.x] + __popc(ballot & ((1u << lane) - 1u));
    for (int w = 0; w < warp; ++w)
        index += warp_hits[w];
    write_step_hit(p, s, h, slot, index, *step_index);
}

//! Live tracks per event: occupied slots plus queued initializers
__global__ void count_event_live_kernel(StateData s, size_type num_events)
{
    size_type const stride = gridDim.x * blockDim.x;
    size_type const tid = thread_slot();
    for (size_type i = tid; i < s.size; i += stride)
    {
        size_type const ev = s.event_id[i];
        if (s.status[i] != status_inactive && ev < num_events)
            atomicAdd(s.event_live + ev, size_type(1));
    }
    size_type const nq = s.counters->num_initializers;
    for (size_type i = tid; i < nq; i += stride)
    {
        size_type const ev = s.initializers[i].event_id;
        if (ev < num_events)
            atomicAdd(s.event_live + ev, size_type(1));
    }
}

//---------------------------------------------------------------------------//
// End of step: vacancies and secondaries
//---------------------------------------------------------------------------//
__global__ __launch_bounds__(block_size) void locate_alive_kernel(StateData s,
                                                                  ScanScratch scr,
                                                                  bool in_place)
{
    __shared__ BlockScanStorage tmp;
    size_type slot = thread_slot();
    bool vacant = false;
    size_type count = 0;
    if (slot < s.size)
    {
        locate_alive(s, slot, &vacant, &count, in_place);
        scr.vacant[slot] = vacant;
        scr.count[slot] = count;
    }
    // Block totals: vacancies with ballot/popc, counts with a block scan
    unsigned int ballot = __ballot_sync(0xffffffffu, vacant);
    __shared__ size_type warp_vac[block_size / 32];
    if ((threadIdx.x & 31) == 0)
        warp_vac[threadIdx.x >> 5] = __popc(ballot);
    size_type total_count;
    block_exclusive_scan(count, tmp, &total_count);
    if (threadIdx.x == 0)
    {
        size_type total_vac = 0;
        for (int w = 0; w < block_size / 32; ++w)
            total_vac += warp_vac[w];
        scr.block_vacant[blockIdx.x] = total_vac;
        scr.block_count[blockIdx.x] = total_count;
    }
}

__global__ __launch_bounds__(1024) void scan_blocks_kernel(StateData s,
                                                           ScanScratch scr,
                                                           StepRecord* log,
                                                           size_type log_capacity,
                                                           size_type* step_index)
{
    // Exclusive scan of the per-block totals by one block of 1024 threads
    __shared__ size_type sh_vac[1024];
    __shared__ size_type sh_cnt[1024];
    __shared__ size_type carry_vac, carry_cnt;
    if (threadIdx.x == 0)
    {
        carry_vac = 0;
        carry_cnt = 0;
    }
    __syncthreads();
    for (size_type base = 0; base < scr.num_blocks; base += 1024)
    {
        size_type i = base + threadIdx.x;
        size_type v = i < scr.num_blocks ? scr.block_vacant[i] : 0;
        size_type c = i < scr.num_blocks ? scr.block_count[i] : 0;
        sh_vac[threadIdx.x] = v;
        sh_cnt[threadIdx.x] = c;
        __syncthreads();
        // Hillis-Steele inclusive scan
        for (int off = 1; off < 1024; off <<= 1)
        {
            size_type av = threadIdx.x >= off ? sh_vac[threadIdx.x - off] : 0;
            size_type ac = threadIdx.x >= off ? sh_cnt[threadIdx.x - off] : 0;
            __syncthreads();
            sh_vac[threadIdx.x] += av;
            sh_cnt[threadIdx.x] += ac;
            __syncthreads();
        }
        if (i < scr.num_blocks)
        {
            scr.block_vacant[i] = carry_vac + sh_vac[threadIdx.x] - v;
            scr.block_count[i] = carry_cnt + sh_cnt[threadIdx.x] - c;
        }
        __syncthreads();
        if (threadIdx.x == 1023)
        {
            carry_vac += sh_vac[1023];
            carry_cnt += sh_cnt[1023];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        Counters& c = *s.counters;
        c.num_vacancies = carry_vac;
        if (carry_cnt > s.initializer_capacity - c.num_initializers)
        {
            // The queue would overflow: this step's secondaries are dropped
            // (the scatter skips them), the queued initializers stay valid
            // and the host reports the overflow
            c.error_flags |= error_initializer_overflow;
            c.num_secondaries = 0;
        }
        else
        {
            c.num_secondaries = carry_cnt;
            c.num_initializers += carry_cnt;
        }
        c.num_alive = s.size - c.num_vacancies;
        StepRecord& r = log[*step_index % log_capacity];
        r.queued = c.num_initializers;
        r.alive = c.num_alive;
        *step_index += 1;
    }
}

__global__ __launch_bounds__(block_size) void scatter_kernel(ParamsData p,
                                                             StateData s,
                                                             ScanScratch scr)
{
    __shared__ BlockScanStorage tmp;
    __shared__ size_type warp_vac[block_size / 32];
    size_type slot = thread_slot();
    bool vacant = false;
    size_type count = 0;
    if (slot < s.size)
    {
        vacant = scr.vacant[slot];
        count = scr.count[slot];
    }
    // Stable position among vacant slots: ballot prefix within the warp plus
    // preceding warps in the block plus preceding blocks
    unsigned int ballot = __ballot_sync(0xffffffffu, vacant);
    int const lane = threadIdx.x & 31;
    int const warp = threadIdx.x >> 5;
    if (lane == 0)
        warp_vac[warp] = __popc(ballot);
    __syncthreads();
    size_type vac_before = 0;
    for (int w = 0; w < warp; ++w)
        vac_before += warp_vac[w];
    vac_before += __popc(ballot & ((1u << lane) - 1u));
    size_type total_count;
    size_type count_before = block_exclusive_scan(count, tmp, &total_count);

    if (slot < s.size)
    {
        Counters const c = *s.counters;
        if (vacant)
        {
            s.vacancies[scr.block_vacant[blockIdx.x] + vac_before] = slot;
        }
        if (!(c.error_flags & error_initializer_overflow))
        {
            process_secondaries(
                p, s, c, slot, scr.block_count[blockIdx.x] + count_before);
        }
    }
}

__global__ void kill_active_kernel(ParamsData p, StateData s)
{
    size_type slot = thread_slot();
    if (slot < s.size && is_track_valid(s.status[slot]))
    {
        apply_errored(p, s, slot);
    }
}

//---------------------------------------------------------------------------//
// Action sort (SortTracksAction): stable counting sort of the track slots by
// action ID in three kernels. Blocks of sort_block_size slots count their
// keys with warp-aggregated shared-memory atomics (match_any + popc); one
// block scans the bin-major [bin][block] counts; the scatter ranks each slot
// among equal keys of its warp (match_any) and of the preceding warps, so
// slots of one action stay in increasing order.
//---------------------------------------------------------------------------//
__device__ __forceinline__ size_type sort_key(StateData const& s,
                                              SortScratch const& srt,
                                              SortKey key,
                                              size_type slot)
{
    size_type const invalid_bin = srt.num_bins - 1;
    if (key == SortKey::start)
    {
        // reindex_status: tracks that are not inactive first (IsNotInactive,
        // TrackSortUtils.cc:71-79); reindex_particle_type: by particle ID
        if (srt.track_order == track_order_reindex_status)
            return s.status[slot] != status_inactive ? 0 : 1;
        size_type const pid = s.particle_id[slot];
        return pid < invalid_bin ? pid : invalid_bin;
    }
    size_type a = (key == SortKey::along_step) ? s.along_step_action[slot]
                                               : s.post_step_action[slot];
    if (!(a < srt.num_actions))
        return invalid_bin;
    if (key == SortKey::along_step && srt.material_actions[0] != invalid_id)
    {
        // Tracks of a material-sorted action by material; later actions
        // after its bins
        size_type const mat = (a == srt.material_actions[0] || a == srt.material_actions[1])
                                  ? min_of(s.material[slot], srt.num_materials - 1)
                                  : 0;
        a = along_bin(srt, a, mat);
    }
    return a;
}

__global__ __launch_bounds__(sort_block_size) void sort_count_kernel(
    StateData s, SortScratch srt, SortKey key)
{
    extern __shared__ size_type hist[];  // [num_bins]
    for (size_type i = threadIdx.x; i < srt.num_bins; i += blockDim.x)
        hist[i] = 0;
    __syncthreads();
    size_type const slot = blockIdx.x * sort_block_size + threadIdx.x;
    bool const valid = slot < s.size;
    size_type const k = valid ? sort_key(s, srt, key, slot) : srt.num_bins;
    unsigned int const peers = __match_any_sync(0xffffffffu, k);
    unsigned int const lane = threadIdx.x & 31u;
    if (valid && (peers & ((1u << lane) - 1u)) == 0)
        atomicAdd(hist + k, static_cast<size_type>(__popc(peers)));
    __syncthreads();
    for (size_type i = threadIdx.x; i < srt.num_bins; i += blockDim.x)
        srt.block_hist[i * srt.num_blocks + blockIdx.x] = hist[i];
}

__global__ __launch_bounds__(1024) void sort_scan_kernel(StateData s,
                                                         SortScratch srt,
                                                         size_type* offsets)
{
    __shared__ size_type warp_sums[32];
    size_type const total = srt.num_bins * srt.num_blocks;
    size_type const per = (total + 1023) / 1024;
    size_type const begin = min_of(total, threadIdx.x * per);
    size_type const end = min_of(total, begin + per);
    size_type sum = 0;
    for (size_type i = begin; i < end; ++i)
        sum += srt.block_hist[i];
    // Block-wide exclusive scan of the per-thread sums
    unsigned int const lane = threadIdx.x & 31u;
    unsigned int const warp = threadIdx.x >> 5;
    size_type incl = sum;
    for (unsigned int off = 1; off < 32; off <<= 1)
    {
        size_type v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off)
            incl += v;
    }
    if (lane == 31)
        warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        size_type const w = warp_sums[lane];
        size_type wi = w;
        for (unsigned int off = 1; off < 32; off <<= 1)
        {
            size_type v = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= off)
                wi += v;
        }
        warp_sums[lane] = wi - w;
    }
    __syncthreads();
    size_type run = warp_sums[warp] + incl - sum;
    for (size_type i = begin; i < end; ++i)
    {
        size_type const c = srt.block_hist[i];
        srt.block_hist[i] = run;
        run += c;
    }
    __syncthreads();
    for (size_type b = threadIdx.x; b < srt.num_bins; b += blockDim.x)
        offsets[b] = srt.block_hist[b * srt.num_blocks];
    if (threadIdx.x == 0)
        offsets[srt.num_bins] = s.size;
}

__global__ __launch_bounds__(sort_block_size) void sort_scatter_kernel(
    StateData s, SortScratch srt, SortKey key)
{
    constexpr unsigned int num_warps = sort_block_size / 32;
    extern __shared__ size_type warp_hist[];  // [num_warps][num_bins]
    size_type const nb = srt.num_bins;
    for (size_type i = threadIdx.x; i < num_warps * nb; i += blockDim.x)
        warp_hist[i] = 0;
    __syncthreads();
    size_type const slot = blockIdx.x * sort_block_size + threadIdx.x;
    bool const valid = slot < s.size;
    size_type const k = valid ? sort_key(s, srt, key, slot) : nb;
    unsigned int const peers = __match_any_sync(0xffffffffu, k);
    unsigned int const lane = threadIdx.x & 31u;
    unsigned int const warp = threadIdx.x >> 5;
    unsigned int const lower = peers & ((1u << lane) - 1u);
    if (valid && lower == 0)
        warp_hist[warp * nb + k] = __popc(peers);
    __syncthreads();
    for (size_type b = threadIdx.x; b < nb; b += blockDim.x)
    {
        size_type acc = 0;
        for (unsigned int w = 0; w < num_warps; ++w)
        {
            size_type const c = warp_hist[w * nb + b];
            warp_hist[w * nb + b] = acc;
            acc += c;
        }
    }
    __syncthreads();
    if (valid)
    {
        size_type const pos = srt.block_hist[k * srt.num_blocks + blockIdx.x]
                              + warp_hist[warp * nb + k] + __popc(lower);
        s.track_slots[pos] = slot;
    }
}

//! Call f(slot) for every slot of the sorted bins [first_bin, end_bin) (or,
//! without offsets, every slot) with a grid-stride loop: a grid of a few
//! blocks per SM covers a range of any length, where a grid sized for the
//! whole state would launch mostly blocks that find no track of the action
//! (the range lives on the device, so the host cannot size the grid to it)
template<class F>
__device__ __forceinline__ void for_each_sorted_slot(StateData const& s,
                                                     size_type const* offsets,
                                                     size_type first_bin,
                                                     size_type end_bin,
                                                     F&& f)
{
    size_type begin = 0;
    size_type end = s.size;
    if (offsets)
    {
        begin = offsets[first_bin];
        end = offsets[end_bin];
    }
    size_type const stride = gridDim.x * blockDim.x;
    for (size_type t = begin + blockIdx.x * blockDim.x + threadIdx.x; t < end; t += stride)
        f(offsets ? s.track_slots[t] : t);
}

// Minimum resident blocks per SM requested for the charged along-step kernel
// (1: the compiler may use up to 255 registers per thread)
#ifndef GBX_ALONG_MIN_BLOCKS
#    define GBX_ALONG_MIN_BLOCKS 1
#endif

// Register cap of the charged along-step kernels (0: none). An SM
// sub-partition holds 16,384 registers, so a cap of 168 per thread keeps 3
// warps resident on each (12 per SM) where 174 keeps 2.
#ifndef GBX_ALONG_MAXNREG
#    define GBX_ALONG_MAXNREG 0
#endif
// The charged kernels come in two instances: blocks of up to 256 threads
// (the kernel's natural register count), and blocks of 512, for which the
// launch bound caps registers at 65536 / 512 = 128 per thread (the compiler
// spills what does not fit)
#if GBX_ALONG_MAXNREG > 0
#    define GBX_ALONG_BOUNDS(THREADS, MINB) __maxnreg__(GBX_ALONG_MAXNREG)
#else
#    define GBX_ALONG_BOUNDS(THREADS, MINB) __launch_bounds__(THREADS, MINB)
#endif
constexpr int along_block_large = 512;

template<AlongKind K, int Threads = block_size>
__global__ GBX_ALONG_BOUNDS(Threads, K == AlongKind::charged ? GBX_ALONG_MIN_BLOCKS : 1) void
along_step_sorted_kernel(ParamsData p,
                         StateData s,
                         size_type const* offsets,
                         size_type first_bin,
                         size_type end_bin)
{
    for_each_sorted_slot(s, offsets, first_bin, end_bin, [&](size_type slot) {
        along_step_impl<K>(p, s, slot);
    });
}

//! Charged along-step in a uniform field over the sorted charged range, as
//! a persistent kernel: each thread takes tracks from a work counter
//! (warp-aggregated), keeps the track's propagation in registers, and runs
//! one field substep per loop iteration, taking the next track as soon as
//! its own finishes. Lanes of a warp thus stay busy on different tracks
//! instead of waiting for the one with the most substeps. Every track runs
//! the same sequence of operations as along_step_impl.
template<int Threads>
__global__ GBX_ALONG_BOUNDS(Threads, 1) void along_charged_persistent_kernel(
    ParamsData p,
    StateData s,
    size_type const* offsets,
    size_type first_bin,
    size_type end_bin,
    size_type* work_counter)
{
    size_type const first = offsets ? offsets[first_bin] : 0;
    size_type const count = offsets ? offsets[end_bin] - first : s.size;
    unsigned int const lane = threadIdx.x & 31u;
    FieldOptions const& opt = p.field_options;
    FieldPropagation fp(opt, UniformFieldEquation{});
    size_type slot = invalid_id;
    bool have = false;
    for (;;)
    {
        if (!have)
        {
            // Claim the next track for every lane that needs one
            unsigned int const need = __activemask();
            unsigned int const rank = __popc(need & ((1u << lane) - 1u));
            unsigned int const leader = __ffs(need) - 1;
            size_type base = 0;
            if (lane == leader)
                base = atomicAdd(work_counter, size_type(__popc(need)));
            base = __shfl_sync(need, base, leader);
            size_type const idx = base + rank;
            if (idx >= count)
                break;
            slot = offsets ? s.track_slots[first + idx] : idx;
            bool charged;
            double start_safety;
            if (!along_prologue<AlongKind::charged>(p, s, slot, &charged, &start_safety))
                continue;
            if (s.step_length[slot] == 0)
            {
                along_epilogue(p, s, slot, true);
                continue;
            }
            GeoTrackView geo(p.geo, s, slot);
            field_setup(p, s, slot, geo, &fp, start_safety);
            have = true;
        }
        GeoTrackView geo(p.geo, s, slot);
        fp.substep(geo);
        if (fp.done())
        {
            field_result(p, s, slot, fp.finish(geo));
            along_epilogue(p, s, slot, true);
            have = false;
        }
    }
}

__global__ __launch_bounds__(block_size) void interact_sorted_kernel(
    ParamsData p,
    StateData s,
    size_type const* offsets,
    size_type first_bin,
    size_type end_bin,
    size_type first_action,
    size_type end_action)
{
    for_each_sorted_slot(s, offsets, first_bin, end_bin, [&](size_type slot) {
        size_type a = s.post_step_action[slot];
        if (a >= first_action && a < end_action)
            interact(p, s, slot, a);
    });
}

__global__ __launch_bounds__(block_size) void boundary_sorted_kernel(
    ParamsData p,
    StateData s,
    size_type const* offsets,
    size_type first_bin,
    size_type end_bin)
{
    for_each_sorted_slot(
        s, offsets, first_bin, end_bin, [&](size_type slot) { boundary_cross(p, s, slot); });
}

__global__ __launch_bounds__(block_size) void tracking_cut_sorted_kernel(
    ParamsData p,
    StateData s,
    size_type const* offsets,
    size_type first_bin,
    size_type end_bin)
{
    for_each_sorted_slot(
        s, offsets, first_bin, end_bin, [&](size_type slot) { tracking_cut(p, s, slot); });
}

//! Bin offsets written by the sort for a key
inline size_type* sort_offsets(LaunchContext const& ctx, SortKey key)
{
    std::size_t const table = std::size_t(ctx.sort.num_bins) + 1;
    return ctx.state.action_offsets + (key == SortKey::step_limit ? table : 0);
}

//! Offsets and bins through which a sorted-range kernel visits its tracks:
//! the action's range of the key's sort; or, for the reindexing orders
//! (shuffle, status, particle type), every slot through the thread -> slot
//! permutation (the shuffle's is fixed when the state is made, the others'
//! are this step's start sort, when it runs)
struct SlotRange
{
    size_type const* offsets;
    size_type first_bin;
    size_type end_bin;
};

inline SlotRange
slot_range(LaunchContext const& ctx, SortKey key, size_type first_bin, size_type end_bin)
{
    unsigned int const order = ctx.params.track_order;
    if (reindexes_all(order))
    {
        bool const permuted = order == track_order_reindex_shuffle || ctx.sort_enabled;
        return {permuted ? sort_offsets(ctx, SortKey::start) : nullptr, 0, ctx.sort.num_bins};
    }
    bool const sorts = key == SortKey::along_step ? sorts_along_step(order)
                                                  : sorts_step_limit(order);
    return {sorts && ctx.sort_enabled ? sort_offsets(ctx, key) : nullptr, first_bin, end_bin};
}

}  // namespace

//---------------------------------------------------------------------------//
// Launchers
//---------------------------------------------------------------------------//
void launch_process_primaries(LaunchContext const& ctx,
                              size_type num_primaries,
                              cudaStream_t stream)
{
    begin_primaries_kernel<<<1, 1, 0, stream>>>(ctx.state, num_primaries);
    size_type n = max_of(num_primaries, ctx.state.size);
    process_primaries_kernel<<<num_blocks_for(n), block_size, 0, stream>>>(
        ctx.state, num_primaries);
}

void launch_generate_primaries(LaunchContext const& ctx,
                               PrimaryGeneratorData const& gen,
                               cudaStream_t stream)
{
    size_type const n = gen.num_events * gen.primaries_per_event;
    generate_primaries_kernel<<<num_blocks_for(n), block_size, 0, stream>>>(
        gen, ctx.state, n);
}

void launch_initialize_tracks(LaunchContext const& ctx, cudaStream_t stream)
{
    if (partitions_by_charge(ctx.params.track_order))
    {
        // InitializeTracksAction with TrackOrder init_charge
        // (InitializeTracksAction.cc:55-95)
        unsigned int const nb = num_blocks_for(ctx.state.size);
        charge_partition_count_kernel<<<nb, block_size, 0, stream>>>(
            ctx.params, ctx.state, ctx.scratch);
        charge_partition_scan_kernel<<<1, 1024, 0, stream>>>(ctx.scratch);
        charge_partition_scatter_kernel<<<nb, block_size, 0, stream>>>(
            ctx.params, ctx.state, ctx.scratch);
        initialize_tracks_charge_kernel<<<ctx.range_blocks, block_size, 0, stream>>>(
            ctx.params, ctx.state);
        finish_initialize_kernel<<<1, 1, 0, stream>>>(
            ctx.state, ctx.log, ctx.log_capacity, ctx.step_index);
        clear_parents_kernel<<<ctx.range_blocks, block_size, 0, stream>>>(ctx.state);
        return;
    }
    if (ctx.partition_slots)
    {
        initialize_tracks_partitioned_kernel<<<num_blocks_for(ctx.state.size),
                                               block_size,
                                               0,
                                               stream>>>(ctx.params, ctx.state);
    }
    else
    {
        initialize_tracks_kernel<<<ctx.range_blocks, block_size, 0, stream>>>(ctx.params,
                                                                            ctx.state);
    }
    finish_initialize_kernel<<<1, 1, 0, stream>>>(
        ctx.state, ctx.log, ctx.log_capacity, ctx.step_index);
}

void launch_pre_step(LaunchContext const& ctx, cudaStream_t stream)
{
    pre_step_kernel<<<num_blocks_for(ctx.state.size), block_size, 0, stream>>>(
        ctx.params, ctx.state);
}


void launch_along_step(LaunchContext const& ctx,
                       size_type action,
                       cudaStream_t stream)
{
    // Each along-step action runs a kernel compiled for that action only,
    // over its sorted range or (sorting off) over all slots; the grid covers
    // the largest range. Sorted and unsorted orders thus run the same code,
    // and a track's result does not depend on the track order.
    ParamsData const& p = ctx.params;
    unsigned int const nb = num_blocks_for(ctx.state.size);
    unsigned int const abs = static_cast<unsigned int>(ctx.along_block_size);
    unsigned int const anb = (ctx.state.size + abs - 1) / abs;
    // Charged along-step grid: up to 2^19 threads (grid-stride beyond), so
    // that a charged range well below the state size does not launch
    // thousands of blocks that find no track
    unsigned int const cnb = min_of(anb, max_of(1u, (1u << 19) / abs));
    size_type cfirst, cend, nfirst, nend;
    along_bins(ctx.sort, p.action_along_step, &cfirst, &cend);
    along_bins(ctx.sort, p.action_along_step_neutral, &nfirst, &nend);
    SlotRange const cr = slot_range(ctx, SortKey::along_step, cfirst, cend);
    SlotRange const nr = slot_range(ctx, SortKey::along_step, nfirst, nend);
    size_type const* offsets = cr.offsets;
    cfirst = cr.first_bin;
    cend = cr.end_bin;
    nfirst = nr.first_bin;
    nend = nr.end_bin;
    if (action == invalid_id || action == p.action_along_step)
    {
        bool const large = abs > static_cast<unsigned int>(block_size);
        if (p.has_field && ctx.persistent_blocks > 0)
        {
            cudaMemsetAsync(ctx.work_counter, 0, sizeof(size_type), stream);
            if (large)
                along_charged_persistent_kernel<along_block_large>
                    <<<ctx.persistent_blocks, abs, 0, stream>>>(
                        p, ctx.state, offsets, cfirst, cend, ctx.work_counter);
            else
                along_charged_persistent_kernel<block_size>
                    <<<ctx.persistent_blocks, abs, 0, stream>>>(
                        p, ctx.state, offsets, cfirst, cend, ctx.work_counter);
        }
        else if (large)
        {
            along_step_sorted_kernel<AlongKind::charged, along_block_large>
                <<<cnb, abs, 0, stream>>>(p, ctx.state, offsets, cfirst, cend);
        }
        else
        {
            along_step_sorted_kernel<AlongKind::charged><<<cnb, abs, 0, stream>>>(
                p, ctx.state, offsets, cfirst, cend);
        }
    }
    if (action == invalid_id || action == p.action_along_step_neutral)
    {
        along_step_sorted_kernel<AlongKind::neutral><<<ctx.range_blocks, block_size, 0, stream>>>(
            p, ctx.state, offsets, nfirst, nend);
    }
}

void launch_discrete_select(LaunchContext const& ctx, cudaStream_t stream)
{
    discrete_select_kernel<<<num_blocks_for(ctx.state.size), block_size, 0, stream>>>(
        ctx.params, ctx.state);
}

void launch_interact(LaunchContext const& ctx, size_type action, cudaStream_t stream)
{
    ParamsData const& p = ctx.params;
    size_type first = action, end = action + 1;
    if (action == invalid_id)
    {
        // All models at once: they are mutually exclusive per slot
        first = p.model_to_action;
        end = p.model_to_action + p.num_models;
    }
    SlotRange const r = slot_range(ctx, SortKey::step_limit, first, end);
    interact_sorted_kernel<<<ctx.range_blocks, block_size, 0, stream>>>(
        p, ctx.state, r.offsets, r.first_bin, r.end_bin, first, end);
}

void launch_boundary(LaunchContext const& ctx, cudaStream_t stream)
{
    ParamsData const& p = ctx.params;
    SlotRange const r
        = slot_range(ctx, SortKey::step_limit, p.action_boundary, p.action_boundary + 1);
    boundary_sorted_kernel<<<ctx.range_blocks, block_size, 0, stream>>>(
        p, ctx.state, r.offsets, r.first_bin, r.end_bin);
}

void launch_tracking_cut(LaunchContext const& ctx, cudaStream_t stream)
{
    ParamsData const& p = ctx.params;
    SlotRange const r = slot_range(
        ctx, SortKey::step_limit, p.action_tracking_cut, p.action_tracking_cut + 1);
    tracking_cut_sorted_kernel<<<ctx.range_blocks, block_size, 0, stream>>>(
        p, ctx.state, r.offsets, r.first_bin, r.end_bin);
}

void launch_calo_tally(LaunchContext const& ctx, cudaStream_t stream)
{
    unsigned int const nb = num_blocks_for(ctx.state.size);
    calo_kernel<<<nb, block_size, 0, stream>>>(ctx.params, ctx.state);
    if (ctx.hits.enabled())
    {
        hits_count_kernel<<<nb, block_size, 0, stream>>>(
            ctx.state, ctx.hits, ctx.hit_block_offsets);
        hits_scan_kernel<<<1, 1024, 0, stream>>>(
            ctx.state, ctx.hit_block_offsets, nb, ctx.hits.capacity);
        hits_scatter_kernel<<<nb, block_size, 0, stream>>>(
            ctx.params, ctx.state, ctx.hits, ctx.hit_block_offsets, ctx.step_index);
    }
}

void launch_extend_from_secondaries(LaunchContext const& ctx, cudaStream_t stream)
{
    unsigned int nb = num_blocks_for(ctx.state.size);
    locate_alive_kernel<<<nb, block_size, 0, stream>>>(
        ctx.state, ctx.scratch, !partitions_by_charge(ctx.params.track_order));
    scan_blocks_kernel<<<1, 1024, 0, stream>>>(
        ctx.state, ctx.scratch, ctx.log, ctx.log_capacity, ctx.step_index);
    scatter_kernel<<<nb, block_size, 0, stream>>>(ctx.params, ctx.state, ctx.scratch);
}

int persistent_along_blocks(int threads_per_block)
{
    int device = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&device) != cudaSuccess
        || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)
               != cudaSuccess
        || (threads_per_block > block_size
                ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                      &per_sm,
                      along_charged_persistent_kernel<along_block_large>,
                      threads_per_block,
                      0)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                      &per_sm,
                      along_charged_persistent_kernel<block_size>,
                      threads_per_block,
                      0))
               != cudaSuccess)
    {
        return 0;
    }
    return sms * per_sm;
}

void launch_count_event_live(LaunchContext const& ctx,
                             size_type num_events,
                             cudaStream_t stream)
{
    cudaMemsetAsync(ctx.state.event_live, 0, sizeof(size_type) * num_events, stream);
    // A grid-stride pass: four blocks per SM of the current device
    static thread_local int sms = 0;
    if (sms == 0)
    {
        int device = 0;
        if (cudaGetDevice(&device) != cudaSuccess
            || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)
                   != cudaSuccess
            || sms <= 0)
        {
            sms = 1;
        }
    }
    count_event_live_kernel<<<4 * sms, block_size, 0, stream>>>(ctx.state, num_events);
}

__global__ __launch_bounds__(block_size) void reseed_kernel(ParamsData p,
                                                            StateData s,
                                                            unsigned int seed,
                                                            unsigned long long event_id)
{
    size_type const slot = thread_slot();
    if (slot < s.size)
    {
        reseed_xorwow_slot(s.rng,
                           p.rng_jump + 32 * 5,
                           seed,
                           event_id * s.size + slot,
                           slot);
    }
}

void launch_reseed(LaunchContext const& ctx,
                   unsigned int seed,
                   unsigned long long event_id,
                   cudaStream_t stream)
{
    reseed_kernel<<<num_blocks_for(ctx.state.size), block_size, 0, stream>>>(
        ctx.params, ctx.state, seed, event_id);
}

void launch_kill_active(LaunchContext const& ctx, cudaStream_t stream)
{
    kill_active_kernel<<<num_blocks_for(ctx.state.size), block_size, 0, stream>>>(
        ctx.params, ctx.state);
}

void launch_sort_tracks(LaunchContext const& ctx, SortKey key, cudaStream_t stream)
{
    SortScratch const& srt = ctx.sort;
    sort_count_kernel<<<srt.num_blocks,
                        sort_block_size,
                        srt.num_bins * sizeof(size_type),
                        stream>>>(ctx.state, srt, key);
    sort_scan_kernel<<<1, 1024, 0, stream>>>(ctx.state, srt, sort_offsets(ctx, key));
    sort_scatter_kernel<<<srt.num_blocks,
                          sort_block_size,
                          (sort_block_size / 32) * srt.num_bins * sizeof(size_type),
                          stream>>>(ctx.state, srt, key);
}

//---------------------------------------------------------------------------//
// Extend-from-secondaries with library-owned scratch
//---------------------------------------------------------------------------//
// The three extend-from-secondaries kernels need 5 bytes of scratch per
// track slot plus 8 bytes per block. This variant takes that scratch from
// one array compiled into the library instead of the stepper's allocation,
// for callers that may not allocate device memory at all. Layout for n
// slots and b = ceil(n / block_size) blocks, each part 256-byte aligned:
//   block_vacant[b] | block_count[b] | count[n] | vacant[n]
namespace
{
constexpr std::size_t align_256(std::size_t bytes)
{
    return (bytes + 255) & ~std::size_t(255);
}

constexpr std::size_t static_scratch_bytes(std::size_t n)
{
    std::size_t const b = (n + block_size - 1) / block_size;
    return 2 * align_256(b * sizeof(size_type))
           + align_256(n * sizeof(size_type)) + align_256(n);
}

// 659,456 bytes for 131,072 track slots
constexpr std::size_t static_scratch_capacity
    = static_scratch_bytes(static_scratch_max_slots);

__device__ __align__(256) unsigned char static_scan_scratch[static_scratch_capacity];

// Device address of static_scan_scratch, looked up once per device
constexpr int static_scratch_max_devices = 64;
std::mutex static_scratch_mutex;
void* static_scratch_address[static_scratch_max_devices] = {};

}  // namespace

unsigned char* static_scratch_for_current_device()
{
    int device = -1;
    if (cudaError_t err = cudaGetDevice(&device); err != cudaSuccess)
    {
        throw std::runtime_error(std::string("cudaGetDevice failed: ")
                                 + cudaGetErrorString(err));
    }
    if (device < 0 || device >= static_scratch_max_devices)
    {
        throw std::runtime_error("static scratch supports device ordinals below "
                                 + std::to_string(static_scratch_max_devices));
    }
    std::lock_guard<std::mutex> lock(static_scratch_mutex);
    if (!static_scratch_address[device])
    {
        void* ptr = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&ptr, static_scan_scratch);
        if (err != cudaSuccess || !ptr)
        {
            throw std::runtime_error(
                std::string("cudaGetSymbolAddress of the static scratch failed: ")
                + cudaGetErrorString(err));
        }
        static_scratch_address[device] = ptr;
    }
    return static_cast<unsigned char*>(static_scratch_address[device]);
}

void launch_extend_from_secondaries_static(LaunchContext const& ctx,
                                           cudaStream_t stream)
{
    size_type const n = ctx.state.size;
    if (n > static_scratch_max_slots)
    {
        throw std::runtime_error(
            "the stepper has " + std::to_string(n)
            + " track slots but the static scratch of extend-from-secondaries "
              "holds at most "
            + std::to_string(static_scratch_max_slots));
    }
    unsigned char* base = static_scratch_for_current_device();
    unsigned int const nb = num_blocks_for(n);
    std::size_t const block_part = align_256(std::size_t(nb) * sizeof(size_type));
    std::size_t const count_part = align_256(std::size_t(n) * sizeof(size_type));

    // Nothing is cleared: locate_alive_kernel writes vacant/count for every
    // slot and both totals for every block before the scan and scatter
    // kernels read them, so the previous call's contents are never used
    ScanScratch scr;
    scr.block_vacant = reinterpret_cast<size_type*>(base);
    scr.block_count = reinterpret_cast<size_type*>(base + block_part);
    scr.count = reinterpret_cast<size_type*>(base + 2 * block_part);
    scr.vacant = base + 2 * block_part + count_part;
    scr.num_blocks = nb;

    locate_alive_kernel<<<nb, block_size, 0, stream>>>(
        ctx.state, scr, !partitions_by_charge(ctx.params.track_order));
    scan_blocks_kernel<<<1, 1024, 0, stream>>>(
        ctx.state, scr, ctx.log, ctx.log_capacity, ctx.step_index);
    scatter_kernel<<<nb, block_size, 0, stream>>>(ctx.params, ctx.state, scr);
}

}  // namespace gbx
