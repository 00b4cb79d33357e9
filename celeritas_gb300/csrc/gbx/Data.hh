// Device-resident parameter tables and the track-state structure of arrays.
//
// Params (read-only, one contiguous device allocation) replace the
// reference's CoreParamsData (src/celeritas/global/CoreTrackData.hh:36-110):
// particles, materials, cutoffs, physics tables, model data and geometry are
// flattened into index-addressed arrays. State replaces CoreStateData
// (src/celeritas/global/CoreTrackData.hh:115-160) as a pure structure of
// arrays: every per-slot field is its own array so that one warp touches one
// contiguous 128-byte line per field.
#pragma once

#include "Random.hh"
#include "Types.hh"

namespace gbx
{
//---------------------------------------------------------------------------//
// Enumerations (values match the reference's enums)
//---------------------------------------------------------------------------//
//! src/celeritas/Types.hh:113-122
enum TrackStatus : std::uint8_t
{
    status_inactive = 0,
    status_initializing = 1,
    status_alive = 2,
    status_errored = 3,
    status_killed = 4,
};

GBX_FORCEINLINE bool is_track_valid(std::uint8_t s)
{
    return s != status_inactive && s != status_errored;
}

//! Track ordering policies (src/celeritas/Types.hh:151-171); the values
//! are the reference's enumerators, all built: 'none', the charge partition
//! of new tracks' slots, the thread -> slot reindexings (shuffle, status,
//! particle type) and the action sorts.
enum TrackOrder : unsigned int
{
    track_order_none = 0,
    track_order_init_charge = 1,
    track_order_reindex_shuffle = 2,
    track_order_reindex_status = 3,
    track_order_reindex_particle_type = 4,
    track_order_reindex_along_step_action = 5,
    track_order_reindex_step_limit_action = 6,
    track_order_reindex_both_action = 7,
};

GBX_FORCEINLINE bool sorts_along_step(unsigned int order)
{
    return order == track_order_reindex_along_step_action
           || order == track_order_reindex_both_action;
}

GBX_FORCEINLINE bool sorts_step_limit(unsigned int order)
{
    return order == track_order_reindex_step_limit_action
           || order == track_order_reindex_both_action;
}

//! Whether the kernels visit every slot through a thread -> slot
//! permutation without action ranges (shuffle, status, particle type)
GBX_FORCEINLINE bool reindexes_all(unsigned int order)
{
    return order == track_order_reindex_shuffle || order == track_order_reindex_status
           || order == track_order_reindex_particle_type;
}

//! Whether new tracks' slots are partitioned by charge (init_charge)
GBX_FORCEINLINE bool partitions_by_charge(unsigned int order)
{
    return order == track_order_init_charge;
}

//! Value grid types (src/celeritas/phys/PhysicsData.hh ValueGridType)
enum ValueGridType : int
{
    vgt_macro_xs = 0,
    vgt_energy_loss = 1,
    vgt_range = 2,
    vgt_size = 3,
};

//! ORANGE-style boundary state (src/orange/OrangeTypes.hh BoundaryResult)
enum BoundaryResult : std::uint8_t
{
    boundary_exiting = 0,
    boundary_reentrant = 1,
};

constexpr int max_processes = 4;  //!< Max processes per particle
constexpr int max_elements = 4;  //!< Max element components per material

//---------------------------------------------------------------------------//
// Tables
//---------------------------------------------------------------------------//
//! Log-uniform energy grid with values; grid energies precomputed on host
struct XsGrid
{
    real_type log_front;  //!< log(E_min)
    real_type log_back;  //!< log(E_max)
    real_type log_delta;  //!< (log_back - log_front) / (size - 1)
    size_type size;
    size_type value;  //!< Offset of values in reals
    size_type energy;  //!< Offset of exp(log_front + i * log_delta) in reals,
                       //!< followed by exp(log_back)
    size_type prime_index;  //!< Values at/after this index are scaled by E
};

//! Nonuniform grid: x and y offsets into reals
struct GenericGrid
{
    size_type x;
    size_type y;
    size_type size;
};

struct ParticleRecord
{
    real_type mass;  //!< [MeV]
    real_type charge;  //!< [e]
    int pdg;
    bool is_antiparticle;
    //! The reference's ParticleId of this particle, which orders particles
    //! by mass, then |PDG|, particles before antiparticles
    //! (ParticleParams::from_import, src/celeritas/phys/ParticleParams.cc:57-71)
    size_type ref_id;
};

struct ElementRecord
{
    int z;
    real_type atomic_mass;  //!< [amu]
    real_type cbrt_z;
    real_type cbrt_zzp;
    real_type log_z;
    real_type coulomb_correction;
    real_type mass_radiation_coeff;
};

struct MaterialRecord
{
    real_type number_density;
    real_type electron_density;
    real_type zeff;
    real_type density;
    real_type rad_length;
    real_type log_mean_exc_energy;
    real_type mean_exc_energy;
    size_type num_elements;
    size_type element[max_elements];
    real_type fraction[max_elements];
};

//! Urban fluctuation parameters per material
struct UrbanFluctRecord
{
    real_type binding_energy[2];
    real_type log_binding_energy[2];
    real_type oscillator_strength[2];
};

//! Per-particle physics process group
struct ProcessGroup
{
    size_type num_processes;
    size_type process[max_processes];  //!< Global process IDs
    //! Models: energy grid (num_models+1 energies) and model IDs per process
    size_type model_energy[max_processes];  //!< Offset in reals
    size_type model_ids[max_processes];  //!< Offset in ints
    size_type num_models[max_processes];
    //! Value grids [vgt][process * num_materials + material] -> grid index
    size_type grid_table[vgt_size];  //!< Offset in ints (invalid_id if none)
    //! Integral approach: energy of max xs per material (offset, or invalid)
    size_type energy_max_xs[max_processes];
    bool use_integral[max_processes];
    size_type eloss_process;  //!< Local process index with dedx/range or -1
    bool has_at_rest;
};

//! Livermore photoelectric data per element
struct LivermoreElement
{
    GenericGrid xs_lo;  //!< size 0 if absent
    GenericGrid xs_hi;
    real_type thresh_lo;
    real_type thresh_hi;
    size_type shells;  //!< Offset of first shell
    size_type num_shells;
};
struct LivermoreShell
{
    real_type binding_energy;
    real_type param[2][6];
    GenericGrid xs;
};

//! Relativistic bremsstrahlung per-element factors
struct RelBremElementRecord
{
    real_type fz;  //!< log(Z)/3 + Coulomb correction
    real_type factor1;  //!< (F_el - f_c) + F_inel / Z
    real_type factor2;  //!< (1 + 1/Z) / 12
    real_type gamma_factor;  //!< 100 m_e / Z^(1/3)
    real_type epsilon_factor;  //!< 100 m_e / Z^(2/3)
};

//! Seltzer-Berger scaled DCS per element
struct SBElementTable
{
    size_type x;  //!< Offset of log-energy grid
    size_type nx;
    size_type y;  //!< Offset of reduced photon energy grid
    size_type ny;
    size_type values;  //!< Offset of [nx][ny] values
    size_type argmax;  //!< Offset (in ints) of per-x argmax over y
};

//! Urban multiple scattering per-material coefficients
struct UrbanMscMaterialRecord
{
    real_type stepmin_coeff[2];
    real_type theta_coeff[2];
    real_type tail_coeff[3];
    real_type tail_corr;
};

//! Urban multiple scattering per-(material, e-/e+) data
struct UrbanMscParMatRecord
{
    real_type scaled_zeff;
    real_type d_over_r;
};

//! Urban multiple scattering parameters
struct UrbanMscParams
{
    bool enabled;
    real_type low_energy_limit;
    real_type high_energy_limit;
    real_type lambda_limit;  //!< PhysicsParamsOptions::lambda_limit
    real_type range_factor;
    real_type safety_factor;
    UrbanMscMaterialRecord const* material;  //!< [material]
    UrbanMscParMatRecord const* par_mat;  //!< [material * 2 + (e+ ? 1 : 0)]
    size_type xs_grids;  //!< Offset in ints: grid index per (material, e-/e+)
};

//! Looping thresholds for charged particles in a field (SimParams)
struct LoopingRecord
{
    size_type max_subthreshold_steps;
    size_type max_steps;
    real_type threshold_energy;
};

//---------------------------------------------------------------------------//
// Geometry: volumes bounded by axis-aligned planes and z-axis cylinders in a
// background world (the ORANGE single-level simple-unit subset used by the
// sampling calorimeter and the CMS-like detector)
//---------------------------------------------------------------------------//
//! Surface types (ORANGE SurfaceType px, py, pz, czc)
enum SurfaceType : int
{
    surf_px = 0,
    surf_py = 1,
    surf_pz = 2,
    surf_czc = 3,  //!< cylinder centered on the z axis
};

//! Surface: a plane (value = position) or a z cylinder (value = radius^2)
struct SurfaceRecord
{
    int type;
    //! sqrt(value) rounded to FP32 for a z cylinder (0 for a plane): only
    //! for conservative reachability bounds, never for a distance
    float radius;
    double value;
    //! sqrt(value) for a z cylinder (0 for a plane), for the mixed build's
    //! safety distance
    double radius_d;
};

//! Volume: conjunction of face senses; inside_sense +1 means the inside is
//! where the surface function is positive (pos > plane, r > radius)
struct VolumeRecord
{
    size_type faces[6];  //!< Surface IDs, sorted
    std::int8_t inside_sense[6];
    size_type num_faces;
    size_type material;
};

//! How points are located among the volumes
enum GeoLocate : int
{
    locate_stack_z = 2,  //!< binary search over boxes layered along z
    locate_scan = 3,  //!< test every volume
};

struct GeoParams
{
    size_type num_surfaces;
    SurfaceRecord const* surfaces;
    size_type num_volumes;  //!< Including exterior (0) and background
    VolumeRecord const* volumes;  //!< Indexed by volume id (exterior/background unused)
    size_type exterior;  //!< Volume id of the exterior (0)
    size_type background;  //!< Volume id of the implicit background
    size_type world_faces[6];  //!< Boundary planes of the world box
    std::int8_t world_sense[6];
    //! Neighbors of each surface: volumes that own it as a face
    size_type const* neighbor_offset;  //!< [num_surfaces + 1]
    size_type const* neighbors;
    int locate;  //!< GeoLocate
    double tol_abs;
    double tol_rel;
    size_type const* volume_material;  //!< [num_volumes], invalid if none
    size_type const* volume_detector;  //!< [num_volumes], invalid if none
    //! Surfaces of each kind sorted by value, ties by ID: planes normal to
    //! x, y and z, then z cylinders ([sorted_offset[k], sorted_offset[k+1])
    //! for kind k = surface type). The background's searches walk them in
    //! the order a ray meets them. sorted_key is each value rounded to FP32
    //! (a cylinder's radius), used only for conservative index bounds.
    size_type sorted_offset[5];
    size_type const* sorted_surfaces;
    float const* sorted_key;
};

//---------------------------------------------------------------------------//
// R-Z magnetic field map (RZMapFieldParamsData,
// src/celeritas/field/RZMapFieldData.hh)
//---------------------------------------------------------------------------//
//! Uniform grid of a field-map axis (UniformGridData::from_bounds)
struct FieldMapGrid
{
    double front;
    double back;
    double delta;
    size_type size;
};

//! Field at a map node [native units]
struct FieldMapElement
{
    double value_z;
    double value_r;
};

//! Field at a map node, rounded to FP32 (mixed-precision stages)
struct FieldMapElementF
{
    float value_z;
    float value_r;
};

//! R-Z map: nodes [z][r] with r fastest
struct RZMapData
{
    FieldMapGrid z;
    FieldMapGrid r;
    FieldMapElement const* values;
    FieldMapElementF const* values_f;
};

//---------------------------------------------------------------------------//
// All parameters
//! Field-driver tuning parameters (FieldDriverOptions,
//! src/celeritas/field/FieldDriverOptions.hh:26-77: the same members and
//! defaults; celer-sim reads them from its 'field_options' input)
struct FieldOptions
{
    double minimum_step = 1.0e-5 * constants::millimeter;
    double delta_chord = 0.25 * constants::millimeter;
    double delta_intersection = 1.0e-4 * constants::millimeter;
    double epsilon_step = 1.0e-5;
    double epsilon_rel_max = 1.0e-3;
    double errcon = 1.0e-4;
    double pgrow = -0.20;
    double pshrink = -0.25;
    double safety = 0.9;
    double max_stepping_increase = 5;
    double max_stepping_decrease = 0.1;
    short max_nsteps = 100;
    short max_substeps = 10;
    static constexpr double initial_step_tol = 1e-6;
    static constexpr double dchord_tol = 1e-5 * constants::millimeter;
    static constexpr double min_chord_shrink = 0.5;

    //! Whether all values are valid (FieldDriverOptions::operator bool)
    bool valid() const
    {
        return minimum_step > 0 && delta_chord > 0 && delta_intersection > minimum_step
               && epsilon_step > 0 && epsilon_step < 1 && epsilon_rel_max > 0
               && pgrow < 0 && pshrink < 0 && safety > 0 && safety < 1
               && max_stepping_increase > 1 && max_stepping_decrease > 0
               && max_stepping_decrease < 1 && max_nsteps > 0 && max_substeps > 0;
    }
};

//---------------------------------------------------------------------------//
struct ParamsData
{
    // Storage: physics tables (FP32 in the mixed-precision build)
    real_type const* reals;
    size_type const* ints;

    // Particles: 0 = e-, 1 = e+, 2 = gamma (same order as the input file)
    size_type num_particles;
    ParticleRecord const* particles;
    size_type electron_id;
    size_type positron_id;
    size_type gamma_id;

    // Materials
    size_type num_materials;
    MaterialRecord const* materials;
    ElementRecord const* elements;
    UrbanFluctRecord const* fluct;
    real_type const* cutoff_energy;  //!< [material * num_particles + particle]

    // Physics
    ProcessGroup const* process_groups;  //!< [particle]
    XsGrid const* grids;
    size_type num_models;
    size_type model_to_action;  //!< Action ID of model 0
    // Scalars (src/celeritas/phys/PhysicsData.hh PhysicsParamsScalars)
    real_type min_range;
    real_type max_step_over_range;
    real_type min_eprime_over_e;
    real_type lowest_electron_energy;
    real_type linear_loss_limit;
    double secondary_stack_factor;
    bool enable_fluct;
    // Hardwired processes
    size_type photoelectric_process;
    size_type annihilation_process;
    real_type photoelectric_table_thresh;
    size_type livermore_model;
    //! Element selection (PhysicsParams::build_model_xs): offset in ints of
    //! [model][particle][material] entries, each the offset in ints of one
    //! CDF grid ID per element component (invalid: no table)
    size_type element_tables;
    size_type eplusgg_model;

    // Model data
    LivermoreElement const* livermore_elements;
    LivermoreShell const* livermore_shells;
    SBElementTable const* sb_tables;
    RelBremElementRecord const* rb_elements;
    bool enable_lpm;

    // Multiple scattering and field
    UrbanMscParams msc;
    bool has_field;
    double field[3];  //!< Uniform field [native units: gauss]
    //! R-Z field map (along-step-rzmap-msc) instead of the uniform field
    bool has_rzmap;
    RZMapData const* rzmap;  //!< In the same memory as the other tables
    LoopingRecord const* looping;  //!< [particle]
    //! XORWOW jump polynomials [2][32][5]: 4^i steps, then 4^i subsequences
    //! of 2^67 steps (XorwowRngParamsData, XorwowRngData.hh:46-47)
    std::uint32_t const* rng_jump;

    // Action IDs (the reference's registration order)
    size_type action_pre_step;
    size_type action_msc_range;
    size_type action_range;
    size_type action_discrete;
    size_type action_integral_rejection;
    size_type action_failure;
    size_type action_along_step;
    size_type action_along_step_neutral;
    size_type action_propagation_limit;
    size_type action_boundary;
    size_type action_tracking_cut;
    // Model actions in model order
    size_type action_moller_bhabha;
    size_type action_seltzer_berger;
    size_type action_rel_brems;
    //! CombinedBremModel ("brems-combined"): Seltzer-Berger below 1 GeV,
    //! relativistic above; invalid unless brem_combined
    size_type action_combined_brems;
    size_type action_livermore_pe;
    size_type action_klein_nishina;
    size_type action_bethe_heitler;
    size_type action_eplusgg;
    // Serving: per-track random streams (each track seeded from its parent's
    // stream, primaries from (seed, event, index)) so that an event's result
    // does not depend on the other events in flight; per-event tallies
    bool rng_per_track;
    bool event_tallies;
    // A field step ending in a reentrant boundary crossing keeps the
    // looping-step count (off: the reference's reset on any non-looping step)
    bool reentrant_looping;
    // Track sorting: policy, sort actions (invalid if absent), action count
    unsigned int track_order;
    size_type action_sort_along;
    size_type action_sort_post;
    size_type action_sort_start;  //!< sort-tracks-status or -start
    size_type num_actions;

    GeoParams geo;

    // Tally
    size_type num_detectors;

    // Field driver (uniform field and R-Z map)
    FieldOptions field_options;
};

//---------------------------------------------------------------------------//
// State (structure of arrays)
//---------------------------------------------------------------------------//
struct Secondary
{
    size_type particle_id;  //!< invalid_id: cut/killed secondary
    real_type energy;
    Vec3<real_type> direction;
};

//! Track initializer (src/celeritas/track/TrackInitData.hh:67-78)
struct TrackInitializer
{
    size_type track_id;
    size_type parent_id;
    size_type event_id;
    double time;
    Real3 pos;
    Real3 dir;
    size_type particle_id;
    real_type energy;
    //! Seed of the track's own random stream (per-track streams only)
    std::uint64_t rng_key;
};

//! Device-resident counters (src/celeritas/track/CoreStateCounters.hh:24-47)
struct Counters
{
    size_type num_vacancies;
    size_type num_initializers;
    size_type num_secondaries;
    size_type num_active;
    size_type num_alive;
    size_type num_generated;
    size_type secondary_stack_size;  //!< Bump allocator top
    size_type num_pending_primaries;
    size_type error_flags;
    size_type num_hits;  //!< Step-output records held on the device
    //! Vacancies taken this step from the front (charged tracks) and the
    //! back (neutral tracks) of the list when slots are partitioned
    size_type num_taken_front;
    size_type num_taken_back;
    size_type pad[4];
};

//---------------------------------------------------------------------------//
// Step output: detector hits (StepCollector / DetectorSteps)
//---------------------------------------------------------------------------//
//! Selected step data (StepSelection, src/celeritas/user/StepData.hh:19-117):
//! the pre- and post-step points and the per-step attributes that
//! DetectorStepOutput holds (src/celeritas/user/DetectorSteps.hh:49-80).
//! The step index, detector and track ID are always recorded.
enum StepSelect : unsigned int
{
    step_pre_time = 1u << 0,
    step_pre_pos = 1u << 1,
    step_pre_dir = 1u << 2,
    step_pre_energy = 1u << 3,
    step_post_time = 1u << 4,
    step_post_pos = 1u << 5,
    step_post_dir = 1u << 6,
    step_post_energy = 1u << 7,
    step_event_id = 1u << 8,
    step_parent_id = 1u << 9,
    step_track_step_count = 1u << 10,
    step_step_length = 1u << 11,
    step_particle = 1u << 12,
    step_energy_deposition = 1u << 13,
    step_select_all = (1u << 14) - 1,
    step_pre_any = step_pre_time | step_pre_pos | step_pre_dir | step_pre_energy,
};

//---------------------------------------------------------------------------//
// Primary generation (PrimaryGenerator, src/celeritas/phys/PrimaryGenerator.cc)
//---------------------------------------------------------------------------//
//! Distribution types (DistributionSelection,
//! src/celeritas/phys/PrimaryGeneratorOptions.hh:21-27)
enum PrimaryDistribution : int
{
    dist_delta = 0,
    dist_isotropic = 1,
    dist_box = 2,
};

//! Generator options (PrimaryGeneratorOptions) for one launch: events
//! [first_event, first_event + num_events) of 'primaries_per_event'
//! primaries each, particles cycling through 'particle_ids'
struct PrimaryGeneratorData
{
    unsigned int seed;
    unsigned int stepper_seed;  //!< Seed of the per-track stream keys
    size_type num_particles;
    size_type particle_ids[8];
    size_type primaries_per_event;
    size_type first_event;
    size_type num_events;
    int energy_dist;
    double energy;
    int position_dist;
    double position[6];
    int direction_dist;
    double direction[3];
};

//! Hit records, one per step of a track in a detector volume: structure of
//! arrays of 'capacity' entries, positions and directions three doubles per
//! record. Arrays of unselected data are null.
struct StepHitsRef
{
    size_type capacity{0};
    unsigned int selection{0};
    //! Drop steps that deposited no energy (StepParamsData::
    //! nonzero_energy_deposition)
    bool nonzero_energy_deposition{true};
    size_type* step{nullptr};  //!< Step iteration of the stepper
    size_type* detector{nullptr};
    size_type* track_id{nullptr};
    size_type* event_id{nullptr};
    size_type* parent_id{nullptr};
    size_type* track_step_count{nullptr};
    size_type* particle{nullptr};
    double* step_length{nullptr};
    double* energy_deposition{nullptr};
    double* pre_time{nullptr};
    double* pre_pos{nullptr};
    double* pre_dir{nullptr};
    double* pre_energy{nullptr};
    double* post_time{nullptr};
    double* post_pos{nullptr};
    double* post_dir{nullptr};
    double* post_energy{nullptr};

    //! Whether hits are collected
    GBX_FORCEINLINE bool enabled() const { return capacity > 0; }
};

struct StateData
{
    size_type size;  //!< Number of track slots

    // Sim
    std::uint8_t* status;
    size_type* track_id;
    size_type* parent_id;
    size_type* event_id;
    size_type* num_steps;
    double* time;
    double* step_length;
    size_type* post_step_action;
    size_type* along_step_action;

    // Particle
    size_type* particle_id;
    real_type* energy;

    // Geometry
    double* pos[3];
    double* dir[3];
    size_type* volume;
    size_type* surface;  //!< Current surface or invalid
    std::int8_t* surface_sense;  //!< Sense of the track relative to surface
    std::uint8_t* boundary;
    double* next_step;
    size_type* next_surface;
    std::int8_t* next_sense;
    std::uint8_t* geo_failed;

    // Material
    size_type* material;

    // Physics
    real_type* interaction_mfp;
    real_type* dedx_range;
    real_type* macro_xs;
    real_type* per_process_xs[max_processes];
    real_type* energy_deposition;
    size_type* secondaries_offset;
    size_type* secondaries_count;
    size_type* element;
    // Multiple scattering step (MscStep) and persistent range (MscRange)
    std::uint8_t* msc_displaced;
    real_type* msc_true_path;
    real_type* msc_geom_path;
    //! log(energy) of the slot's energy 'key' (FP64 build), kept across the
    //! step's actions; a NaN key matches no energy
    real_type* log_energy_key;
    real_type* log_energy_value;
    //! init_charge: the new tracks' initializers (offsets into the last
    //! num_new of the list), neutral ones first, each group in list order
    size_type* init_indices;
    real_type* msc_alpha;
    real_type* msc_range_init;
    real_type* msc_range_factor;
    real_type* msc_limit_min;
    // Field looping counter
    size_type* num_looping_steps;

    // RNG
    RngStateRef rng;

    // Track initialization
    size_type* vacancies;
    size_type* secondary_counts;
    size_type* parents;
    TrackInitializer* initializers;
    size_type initializer_capacity;
    size_type* track_counters;  //!< Per-event next track ID
    size_type max_events;

    // Secondary stack
    Secondary* secondaries;
    size_type secondary_capacity;

    // Step gather: detector ID at pre-step
    size_type* detector;
    // Step output: pre-step point of slots in a detector volume, per slot
    // (positions and directions three doubles per slot); null unless hits
    // with that datum are collected
    double* pre_time;
    double* pre_pos;
    double* pre_dir;
    double* pre_energy;
    // Tally: energy deposition per detector (FP64 accumulation)
    double* calo_edep;

    // Primaries staging
    TrackInitializer* primaries;
    size_type primary_capacity;

    // Per-event energy deposition in detectors and live-track counts
    // ([max_events]; null without per-event tallies)
    double* event_edep;
    size_type* event_live;
    // Per-event energy deposition of each detector ([max_events][detectors],
    // event-major; null without per-event tallies)
    double* event_det_edep;

    // Action-sorted thread -> slot indirection (CoreStateData::track_slots)
    // and the first thread of each action bin, one table per sort key:
    // along-step sort at [0, num_actions + 2), step-limit sort after it.
    // The last bin of a table holds slots whose action is invalid.
    size_type* track_slots;
    size_type* action_offsets;

    Counters* counters;
};

}  // namespace gbx
