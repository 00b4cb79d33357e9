/*
 * C ABI of the GB300 electromagnetic-shower stepping loop.
 *
 * The boundary mirrors the reference's plugin API for the stepping loop:
 *
 *   - gbx_params_*   <-> celeritas::CoreParams (src/celeritas/global/CoreParams.hh:68-172)
 *                        built as in celer-sim's Runner::build_core_params
 *                        (app/celer-sim/Runner.cc:281-446)
 *   - gbx_stepper_*  <-> celeritas::Stepper<MemSpace::device>
 *                        (src/celeritas/global/Stepper.hh:43-201): operator(),
 *                        operator()(Span<Primary const>), kill_active
 *   - gbx_stepper_launch_action
 *                    <-> CoreStepActionInterface::step(CoreParams const&,
 *                        CoreStateDevice&) (src/corecel/sys/ActionInterface.hh:176-186),
 *                        one call per registered action ID
 *   - gbx_primary    <-> celeritas::Primary (src/celeritas/phys/Primary.hh:23-31)
 *   - gbx_step_result <-> celeritas::StepperResult (src/celeritas/global/Stepper.hh:61-70)
 *
 * All functions return 0 on success and nonzero on failure; the message of
 * the last failure on the calling thread is available from gbx_last_error().
 * Plain pointers and sizes only: no C++ or framework types cross the ABI.
 */
#ifndef CELERITAS_GB300_H
#define CELERITAS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbx_params_s gbx_params;
typedef struct gbx_stepper_s gbx_stepper;

/* A primary particle (celeritas::Primary): PDG code, kinetic energy [MeV],
 * position [cm], unit direction, time [s], event index */
typedef struct
{
    int pdg;
    double energy;
    double pos[3];
    double dir[3];
    double time;
    unsigned int event_id;
} gbx_primary;

/* Track counts after a step (celeritas::StepperResult) */
typedef struct
{
    unsigned int generated;
    unsigned int queued;
    unsigned int active;
    unsigned int alive;
} gbx_step_result;

/* Message describing the last error on this thread ("" if none) */
const char* gbx_last_error(void);

/* Track ordering policies (celeritas::TrackOrder, src/celeritas/Types.hh:151-171,
 * with the reference's enumerator values); only these are supported */
enum
{
    GBX_TRACK_ORDER_NONE = 0,
    GBX_TRACK_ORDER_REINDEX_ALONG_STEP_ACTION = 5,
    GBX_TRACK_ORDER_REINDEX_STEP_LIMIT_ACTION = 6,
    GBX_TRACK_ORDER_REINDEX_BOTH_ACTION = 7
};

/* Field-driver options (FieldDriverOptions,
 * src/celeritas/field/FieldDriverOptions.hh:26-77; celer-sim's
 * 'field_options'), lengths in cm; gbx_field_driver_options_default fills
 * the reference's defaults. */
typedef struct
{
    double minimum_step;
    double delta_chord;
    double delta_intersection;
    double epsilon_step;
    double epsilon_rel_max;
    double errcon;
    double pgrow;
    double pshrink;
    double safety;
    double max_stepping_increase;
    double max_stepping_decrease;
    int max_nsteps;
    int max_substeps;
} gbx_field_driver_options;
void gbx_field_driver_options_default(gbx_field_driver_options* options);

/* Physics options (the RunnerInput field / physics_options / track_order
 * knobs, app/celer-sim/RunnerInput.hh:41-141): a uniform magnetic field in
 * tesla (all zero: straight-line transport, along-step-general-linear;
 * otherwise along-step-uniform-msc), Urban multiple scattering for e-/e+,
 * and the track order (the reference's TrackOrder values: 0 none, 1
 * init_charge, 2 reindex_shuffle, 3 reindex_status, 4
 * reindex_particle_type, 5-7 the action sorts). The reindexing orders 2-4
 * change which thread visits which slot, not the results; 3 and 4 register
 * sort-tracks-status and sort-tracks-start. An action-sorting order registers the
 * reference's sort-tracks-post-step and/or sort-tracks-along-step actions
 * (after extend-from-secondaries, CoreParams.cc:258-283) and launches the
 * sorted actions over their ranges of action-sorted track slots;
 * init_charge registers none and lets neutral and charged new tracks fill
 * the two ends of the vacant slots (InitTracksExecutor.hh:71-108). */
typedef struct
{
    double field_tesla[3];
    int msc;
    unsigned int track_order;
    /* Serving options, without counterparts in the reference. Nonzero
     * rng_per_track gives every track its own random stream, seeded from its
     * parent's stream (primaries: from the stepper seed, the event ID and
     * the primary's index within its event), so that an event's result does
     * not depend on which other events share the stepper. Nonzero
     * event_tallies accumulates detector energy deposition per event. */
    int rng_per_track;
    int event_tallies;
    /* Nonzero: a field-propagation step that ends on a boundary which the
     * track re-enters at once (ORANGE's reentrant crossing, back into the
     * volume it came from) keeps a looping track's looping-step count
     * instead of resetting it. Without counterpart in the reference, whose
     * looping cut (PropagationApplier,
     * src/celeritas/global/alongstep/detail/PropagationApplier.hh:147-170)
     * resets the count on any step that is not looping: a low-energy
     * electron circling in vacuum with its orbit grazing a surface then
     * never reaches the cut, and celer-sim ends such a run only by its
     * global step limit (app/celer-sim/Transporter.cc:135-150). Zero keeps
     * the reference's behaviour. */
    int reentrant_looping;
    /* Path of an R-Z magnetic field map (NULL or empty: none; excludes
     * field_tesla): along-step-rzmap-msc with the map interpolated as
     * RZMapField does (src/celeritas/field/RZMapField.hh), in place of
     * along-step-uniform-msc. Text: 'rzmap num_z num_r min_z max_z min_r
     * max_r' [cm], then 'Bz Br' [tesla] per node, z-major ([Z][R], the
     * order of RZMapFieldInput, src/celeritas/field/RZMapFieldInput.hh). */
    const char* rz_field_file;
    /* RunnerInput::brem_combined (app/celer-sim/RunnerInput.hh:120):
     * nonzero registers the combined bremsstrahlung model
     * (CombinedBremModel, "brems-combined": Seltzer-Berger below 1 GeV,
     * relativistic above) in place of "brems-sb" and "brems-rel"; every
     * material must then hold a single element (otherwise an error, as
     * PhysicsParams.cc:660-668 raises). */
    int brem_combined;
    /* RunnerInput::secondary_stack_factor: secondaries per track slot held
     * by the per-step secondary stack (PhysicsParams.hh:250,501-502); zero
     * takes the reference's default, 3. */
    double secondary_stack_factor;
    /* Field-driver options; NULL: the reference's defaults. Rejected unless
     * valid (FieldDriverOptions::operator bool). */
    const gbx_field_driver_options* field_options;
    /* RunnerInput::initializer_capacity (TrackInitParams' capacity): the
     * pending-track queue of each stepper created from these parameters;
     * zero: 16 per track slot (at least 2^20). */
    unsigned int initializer_capacity;
} gbx_params_options;

/* Build problem parameters from a physics input file and a named geometry
 * ("calo": 50-layer Pb/lAr sampling calorimeter); 'options' may be NULL
 * (no field, no MSC). Replaces Runner::build_core_params
 * (app/celer-sim/Runner.cc:281-446). */
int gbx_params_create(const char* physics_file,
                      const char* geometry,
                      const gbx_params_options* options,
                      gbx_params** out);
void gbx_params_destroy(gbx_params* params);
/* Registered actions, in ID order (ActionRegistry::id_to_label,
 * src/corecel/sys/ActionRegistry.hh:58-92) */
int gbx_params_num_actions(const gbx_params* params, unsigned int* num);
int gbx_params_action_label(const gbx_params* params,
                            unsigned int action_id,
                            char* buf,
                            size_t buf_size);
/* Energy-deposition detectors (SimpleCalo volume labels,
 * src/celeritas/user/SimpleCalo.hh:40-86) */
int gbx_params_num_detectors(const gbx_params* params, unsigned int* num);
int gbx_params_detector_label(const gbx_params* params,
                              unsigned int detector,
                              char* buf,
                              size_t buf_size);

/* Create a stepper with its own device state and CUDA stream
 * (Stepper(StepperInput), src/celeritas/global/Stepper.cc:66-87).
 * 'use_graph' replays steps without primaries from a captured CUDA graph. */
int gbx_stepper_create(gbx_params* params,
                       unsigned int num_track_slots,
                       unsigned int seed,
                       int use_graph,
                       gbx_stepper** out);
void gbx_stepper_destroy(gbx_stepper* stepper);

/* Take one step, inserting 'num_primaries' primaries first if nonzero
 * (Stepper::operator()(Span<Primary const>) / operator()()) */
int gbx_stepper_step(gbx_stepper* stepper,
                     const gbx_primary* primaries,
                     size_t num_primaries,
                     gbx_step_result* result);

/* Step until no tracks are queued or alive, or 'max_steps' steps; writes up
 * to 'capacity' per-step results and the number of steps taken. Host reads
 * happen every 'batch' steps only. (celer-sim Transporter loop,
 * app/celer-sim/Transporter.cc:139-162) */
int gbx_stepper_run(gbx_stepper* stepper,
                    unsigned int max_steps,
                    unsigned int batch,
                    gbx_step_result* results,
                    size_t capacity,
                    unsigned int* num_steps);

/* Launch the kernel(s) of one registered step action on the stepper's
 * stream (CoreStepActionInterface::step for MemSpace::device) */
int gbx_stepper_launch_action(gbx_stepper* stepper, unsigned int action_id);

/* Stage primaries for the next extend-from-primaries action
 * (ExtendFromPrimariesAction::insert, src/celeritas/track/ExtendFromPrimariesAction.cc:103-190) */
int gbx_stepper_insert_primaries(gbx_stepper* stepper,
                                 const gbx_primary* primaries,
                                 size_t num_primaries);

/* Distributions of the primary generator (DistributionSelection,
 * src/celeritas/phys/PrimaryGeneratorOptions.hh:21-27, same values) */
enum
{
    GBX_DIST_DELTA = 0,
    GBX_DIST_ISOTROPIC = 1,
    GBX_DIST_BOX = 2
};

/* Primary generator options (PrimaryGeneratorOptions,
 * src/celeritas/phys/PrimaryGeneratorOptions.hh:47-73, as celer-sim reads
 * them): 'num_pdg' PDG codes cycled over the primaries of each event;
 * energy [MeV]: delta (1 parameter); position [cm]: delta (x, y, z) or box
 * (lower x, y, z, then upper x, y, z); direction: delta (a unit vector) or
 * isotropic (no parameter). */
typedef struct
{
    unsigned int seed;
    int pdg[8];
    unsigned int num_pdg;
    unsigned int num_events;
    unsigned int primaries_per_event;
    int energy_distribution;
    double energy[1];
    int position_distribution;
    double position[6];
    int direction_distribution;
    double direction[3];
} gbx_primary_generator_options;

/* Sample the primaries of events [first_event, first_event + num_events)
 * on the device, into the stepper's staging buffer, for the next
 * gbx_stepper_step (PrimaryGenerator::operator() for each event,
 * src/celeritas/phys/PrimaryGenerator.cc:63-83): no host memory and no
 * host-to-device copy. Each primary samples from its own XORWOW stream keyed
 * by the seed, its event and its index in the event, so the sequence is not
 * the reference's mt19937 one; the distributions are. The events must not
 * have primaries yet. Invalid options fail with the reference's messages. */
int gbx_stepper_generate_primaries(gbx_stepper* stepper,
                                   const gbx_primary_generator_options* options,
                                   unsigned int first_event);

/* Kill all active tracks (Stepper::kill_active) */
int gbx_stepper_kill_active(gbx_stepper* stepper);

/* Reseed the random state of every track slot for an event and restart the
 * per-event track IDs (Stepper::reseed(UniqueEventId),
 * src/celeritas/global/Stepper.hh:111,175 and Stepper.cc:194-201): slot i
 * gets the XORWOW state of the stepper's seed advanced
 * event_id * num_track_slots + i subsequences of 2^67 draws
 * (src/celeritas/random/RngReseed.cc:27-47). */
int gbx_stepper_reseed(gbx_stepper* stepper, unsigned long long event_id);

/* Wait for all work on the stepper's stream */
int gbx_stepper_synchronize(gbx_stepper* stepper);

/* The stepper's CUDA stream (a cudaStream_t) for event timing by callers */
int gbx_stepper_stream(gbx_stepper* stepper, void** stream);

/* Number of kernel nodes in one graph-replayed step (builds the graph) */
int gbx_stepper_step_kernels(gbx_stepper* stepper, unsigned int* num_kernels);

/* Time every action's kernels with CUDA events on the stepper's stream
 * (StepperInput::action_times, src/celeritas/global/Stepper.hh:43-55; steps
 * are then launched eagerly instead of from the CUDA graph) */
int gbx_stepper_set_action_times(gbx_stepper* stepper, int enable);
/* Accumulated milliseconds and launch counts per action ID ('capacity'
 * entries, indexed by action ID); the counters are then reset */
int gbx_stepper_action_times(gbx_stepper* stepper,
                             double* milliseconds,
                             unsigned int* launches,
                             size_t capacity);

/* Accumulated energy deposition per detector [MeV] (SimpleCalo
 * calc_total_energy_deposition) and its reset */
int gbx_stepper_energy_deposition(gbx_stepper* stepper,
                                  double* out,
                                  size_t num_detectors);
int gbx_stepper_clear_energy_deposition(gbx_stepper* stepper);

/* Copy one named state array between host and device (direction > 0:
 * host -> device). Names: status, track_id, parent_id, event_id, num_steps,
 * time, step_length, post_step_action, along_step_action, particle_id,
 * energy, pos_x|y|z, dir_x|y|z, volume, surface, surface_sense, boundary,
 * material, interaction_mfp, dedx_range, macro_xs, per_process_xs_0..3,
 * energy_deposition, secondaries_offset, secondaries_count, element,
 * rng (6 x slots words), vacancies, parents, counters, initializers,
 * secondaries, detector. Used by tests to load a state snapshot, run one
 * action and read the result. */
int gbx_stepper_copy_state(gbx_stepper* stepper,
                           const char* field,
                           void* host,
                           size_t nbytes,
                           int direction);

/* Bytes per element of a named state array and the number of elements */
int gbx_stepper_state_info(gbx_stepper* stepper,
                           const char* field,
                           size_t* elem_bytes,
                           size_t* count);

/* Tracks in each action's range of the stepper's last action sort, indexed
 * by action ID: key 0 the sort by along-step action (before the along-step
 * kernels), 1 the sort by step-limit action (before the interactions);
 * num_actions must equal gbx_params_num_actions. Synchronizes the stepper's
 * stream. A profiler's view of what SortTracksAction partitioned
 * (src/celeritas/track/SortTracksAction.cc); no counterpart in the
 * reference's API. */
int gbx_stepper_sorted_action_sizes(gbx_stepper* stepper,
                                    int key,
                                    unsigned int* sizes,
                                    size_t num_actions);

/* Live tracks per event, for events [0, num_events): occupied track slots
 * plus queued track initializers; synchronizes the stepper's stream. A
 * serving loop reads it to detect completed events. No counterpart in the
 * reference. */
int gbx_stepper_event_live(gbx_stepper* stepper,
                           unsigned int* counts,
                           size_t num_events);

/* Energy deposited in detectors per event [MeV], for events
 * [0, num_events), with the event_tallies option; 'clear' resets the
 * tallies after reading. No counterpart in the reference. */
int gbx_stepper_event_energy_deposition(gbx_stepper* stepper,
                                        double* out,
                                        size_t num_events,
                                        int clear);

/* Energy deposited in each detector per event [MeV], for events
 * [first_event, first_event + num_events), with the event_tallies option:
 * 'out' holds num_events x (number of detectors) values, event-major, in
 * the detector order of gbx_params_detector_label; 'clear' resets those
 * tallies after reading. The per-event form of the SimpleCalo tally
 * (src/celeritas/user/SimpleCalo.hh:40-90 keeps one sum per detector for
 * the whole run); no counterpart in the reference. */
int gbx_stepper_event_detector_energy_deposition(gbx_stepper* stepper,
                                                 double* out,
                                                 unsigned int first_event,
                                                 size_t num_events,
                                                 int clear);

/* Step data recorded for each hit (StepSelection's fields,
 * src/celeritas/user/StepData.hh:19-117, as DetectorStepOutput holds them,
 * src/celeritas/user/DetectorSteps.hh:49-80). The step index, detector and
 * track ID of a hit are always recorded. */
enum
{
    GBX_STEP_PRE_TIME = 1u << 0,
    GBX_STEP_PRE_POS = 1u << 1,
    GBX_STEP_PRE_DIR = 1u << 2,
    GBX_STEP_PRE_ENERGY = 1u << 3,
    GBX_STEP_POST_TIME = 1u << 4,
    GBX_STEP_POST_POS = 1u << 5,
    GBX_STEP_POST_DIR = 1u << 6,
    GBX_STEP_POST_ENERGY = 1u << 7,
    GBX_STEP_EVENT_ID = 1u << 8,
    GBX_STEP_PARENT_ID = 1u << 9,
    GBX_STEP_TRACK_STEP_COUNT = 1u << 10,
    GBX_STEP_STEP_LENGTH = 1u << 11,
    GBX_STEP_PARTICLE = 1u << 12,
    GBX_STEP_ENERGY_DEPOSITION = 1u << 13,
    GBX_STEP_ALL = (1u << 14) - 1
};

/* Hit records in the caller's host memory: each non-null array holds
 * 'capacity' entries (positions and directions three doubles per record).
 * 'step' is the stepper's step iteration of the hit; 'particle' is the
 * reference's ParticleId; energies in MeV, times in seconds, lengths in cm.
 * The records of a step come in track-slot order, as copy_steps writes
 * them (src/celeritas/user/DetectorSteps.cc). */
typedef struct
{
    size_t capacity;
    unsigned int* step;
    unsigned int* detector;
    unsigned int* track_id;
    unsigned int* event_id;
    unsigned int* parent_id;
    unsigned int* track_step_count;
    unsigned int* particle;
    double* step_length;
    double* energy_deposition;
    double* pre_time;
    double* pre_pos;
    double* pre_dir;
    double* pre_energy;
    double* post_time;
    double* post_pos;
    double* post_dir;
    double* post_energy;
} gbx_step_hits;

/* Collect the hits of every step: a StepCollector with one step interface
 * over the detector volumes of the energy-deposition tally
 * (src/celeritas/user/StepCollector.hh:33-80, StepInterface.hh:40-75), whose
 * process_steps copies the hits out (copy_steps,
 * src/celeritas/user/DetectorSteps.hh:83-90). 'selection' is a mask of
 * GBX_STEP_* bits; nonzero 'nonzero_energy_deposition' drops steps without
 * deposition (StepInterface::Filters). Hits accumulate on the device, up to
 * 'capacity' records, between calls of gbx_stepper_read_step_output; zero
 * capacity turns the output off. Allocates the device buffers here, never
 * inside the step loop. */
int gbx_stepper_set_step_output(gbx_stepper* stepper,
                                unsigned int selection,
                                int nonzero_energy_deposition,
                                size_t capacity);

/* Copy the hits held on the device into 'out' (synchronizes the stream),
 * write their number to 'num_hits' and empty the device buffers. Fails if
 * the device buffers overflowed since the last read (they are emptied; the
 * steps' other results are unaffected) or if 'out->capacity' is below the
 * number held (they are kept). */
int gbx_stepper_read_step_output(gbx_stepper* stepper,
                                 const gbx_step_hits* out,
                                 size_t* num_hits);

/* Launch tuning of a stepper, for an autotuner (no counterpart in the
 * reference, whose block sizes and sort policy are build and run options):
 *   "along_block_size"  threads per block of the charged along-step (64, 128,
 *                       256, or 512 with registers capped at 128 per thread)
 *   "along_persistent"  1: charged along-step as a persistent kernel that
 *                       interleaves field substeps of different tracks
 *   "sort_threshold"    with an action-sorting track order, sort only in
 *                       steps that start with at least this many live
 *                       tracks (0: always)
 *   "sort"              0: action sorts off (each action kernel visits
 *                       every slot), 1: on; reset by the sort threshold
 *   "sort_material"     bit 0: the along-step sort orders the charged
 *                       tracks by material too, so that warps of the charged
 *                       kernel hold tracks of one material; bit 1: the
 *                       neutral tracks (0-3)
 *   "partition_slots"   1: new charged tracks take the lowest vacant slots
 *                       and neutral ones the highest, so the sorted ranges
 *                       of the along-step kernels cover mostly contiguous
 *                       slots (only with rng_per_track; error otherwise)
 * Results do not depend on these settings (in the mixed build, the
 * 512-thread instances may round an FP32 deposit differently in its last
 * bit, their compiled arithmetic being contracted separately; with
 * partitioned slots the per-event tallies sum in another order). Setting
 * one drops the captured step graphs. */
int gbx_stepper_set_tuning(gbx_stepper* stepper, const char* name, long long value);
int gbx_stepper_get_tuning(gbx_stepper* stepper, const char* name, long long* value);

/* Stepper::warm_up (src/celeritas/global/Stepper.hh:99, Stepper.cc:105-115):
 * run one step over the empty state so that every kernel is loaded and the
 * step graph of each sort state is captured before the first timed step
 * (celer-sim's RunnerInput::warm_up). Fails if tracks are active or
 * queued; leaves the state, counters and tallies unchanged. */
int gbx_stepper_warm_up(gbx_stepper* stepper);

/* Number of device allocations (cudaMalloc calls) this library has made so
 * far, over all devices: parameter and state storage, step-output buffers
 * and gbx_libm_evaluate's buffers. A caller can read it around a call to
 * check that the call allocated nothing. No counterpart in the reference. */
int gbx_device_allocations(unsigned long long* count);

/* Largest stepper (track slots) accepted by
 * gbx_stepper_extend_from_secondaries_static */
#define GBX_STATIC_SCRATCH_MAX_SLOTS 131072

/* The extend-from-secondaries step action (what gbx_stepper_launch_action
 * runs for that action ID) with its scan scratch taken from a fixed array
 * compiled into this library, so that the call allocates no device memory.
 * This entry point has no counterpart in the reference.
 *
 * It is for callers that launch the end-of-step compaction from code that
 * may not allocate device memory: a host framework that owns all device
 * memory through its own fixed pool and forbids cudaMalloc after start-up
 * (an allocation there would bypass the pool's accounting, may synchronise
 * the device, and can fail once the pool has claimed the memory).
 *
 * - The scratch is 659,456 bytes and fits steppers of at most
 *   GBX_STATIC_SCRATCH_MAX_SLOTS track slots; larger ones are rejected with
 *   an error and nothing is launched.
 * - The array's device address is looked up (cudaGetSymbolAddress) once
 *   per device: gbx_stepper_create does it for steppers small enough, with
 *   that device current; if that was skipped, the first call on the device
 *   does it, and that first call should then come before any stream
 *   capture. The stepper's device must be current at every call (checked:
 *   another current device is an error).
 * - Every call on a device shares the one array and leaves its contents
 *   behind. Each call writes every scratch element before reading it, so
 *   nothing needs clearing; but calls that overlap on the GPU (two steppers
 *   on different streams) race on the array and corrupt each other.
 * - Kernels are launched on the stepper's stream; the call does not wait
 *   for them. */
int gbx_stepper_extend_from_secondaries_static(gbx_stepper* stepper);

/* Elementary functions of the FP64 stepping loop (correctly rounded; see
 * celeritas_gb300/csrc/gbx/Libm.hh), evaluated on the device: y[i] = f(x[i])
 * for host arrays of n doubles, copied to and from the current device.
 * No counterpart in the reference, whose host and device builds call their
 * platforms' own libraries; this entry point lets a caller (or a test) check
 * that the device results equal the host ones bit for bit. */
enum
{
    GBX_LIBM_EXP = 0,
    GBX_LIBM_LOG = 1,
    GBX_LIBM_SIN = 2,
    GBX_LIBM_COS = 3,
    GBX_LIBM_TANH = 4,
    GBX_LIBM_LOG1P = 5,
    GBX_LIBM_EXPM1 = 6,
    GBX_LIBM_CBRT = 7
};
int gbx_libm_evaluate(int function, const double* x, double* y, size_t n);

#ifdef __cplusplus
}
#endif

#endif /* CELERITAS_GB300_H */
