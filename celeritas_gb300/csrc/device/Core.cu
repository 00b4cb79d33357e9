// Device-side implementation of the host API: parameter upload, state
// allocation, the registered step actions and the graph-replayed stepper.
#include "../host/Core.hh"
#include "../gbx/Random.hh"

#include <algorithm>
#include <random>
#include <atomic>
#include <cstring>
#include <stdexcept>

#include "../host/HostState.hh"

namespace gbx
{
namespace
{
void check(cudaError_t err, char const* what)
{
    if (err != cudaSuccess)
    {
        throw std::runtime_error(std::string(what) + ": "
                                 + cudaGetErrorString(err));
    }
}
#define GBX_CUDA(call) ::gbx::check((call), #call)

//! Packs host arrays into one aligned byte buffer
class Packer
{
  public:
    template<class T>
    std::size_t add(std::vector<T> const& v)
    {
        return this->add_bytes(v.data(), v.size() * sizeof(T));
    }
    std::size_t add_bytes(void const* data, std::size_t nbytes)
    {
        std::size_t off = (bytes_.size() + 255) & ~std::size_t(255);
        bytes_.resize(off + std::max<std::size_t>(nbytes, 1));
        if (nbytes)
            std::memcpy(bytes_.data() + off, data, nbytes);
        return off;
    }
    std::vector<unsigned char> const& bytes() const { return bytes_; }

  private:
    std::vector<unsigned char> bytes_;
};

//! Computes aligned offsets for a device allocation
class Layout
{
  public:
    std::size_t reserve(std::size_t nbytes)
    {
        std::size_t off = (size_ + 255) & ~std::size_t(255);
        size_ = off + std::max<std::size_t>(nbytes, 1);
        return off;
    }
    std::size_t size() const { return size_; }

  private:
    std::size_t size_{0};
};

//---------------------------------------------------------------------------//
// Actions
//---------------------------------------------------------------------------//
class KernelAction : public CoreStepActionInterface, public ConcreteAction
{
  public:
    using Launch = void (*)(CoreParams const&, CoreState&, ActionId);
    KernelAction(ActionId id,
                 std::string label,
                 std::string description,
                 StepActionOrder order,
                 Launch launch)
        : ConcreteAction(id, std::move(label), std::move(description))
        , order_(order)
        , launch_(launch)
    {
    }
    StepActionOrder order() const final { return order_; }
    void step(CoreParams const& params, CoreState& state) const final
    {
        if (launch_)
            launch_(params, state, this->action_id());
    }

  private:
    StepActionOrder order_;
    Launch launch_;
};

void step_primaries(CoreParams const&, CoreState& state, ActionId)
{
    if (size_type n = state.pending_primaries())
    {
        launch_process_primaries(state.context(), n, state.stream());
        state.clear_pending_primaries();
    }
}
void step_init(CoreParams const&, CoreState& state, ActionId)
{
    launch_initialize_tracks(state.context(), state.stream());
}
void step_pre(CoreParams const&, CoreState& state, ActionId)
{
    launch_pre_step(state.context(), state.stream());
}
void step_along(CoreParams const&, CoreState& state, ActionId id)
{
    launch_along_step(state.context(), id, state.stream());
}
void step_discrete(CoreParams const&, CoreState& state, ActionId)
{
    launch_discrete_select(state.context(), state.stream());
}
void step_model(CoreParams const&, CoreState& state, ActionId id)
{
    launch_interact(state.context(), id, state.stream());
}
void step_boundary(CoreParams const&, CoreState& state, ActionId)
{
    launch_boundary(state.context(), state.stream());
}
void step_cut(CoreParams const&, CoreState& state, ActionId)
{
    launch_tracking_cut(state.context(), state.stream());
}
void step_calo(CoreParams const&, CoreState& state, ActionId)
{
    launch_calo_tally(state.context(), state.stream());
}
void step_secondaries(CoreParams const&, CoreState& state, ActionId)
{
    launch_extend_from_secondaries(state.context(), state.stream());
}
void step_sort_along(CoreParams const&, CoreState& state, ActionId)
{
    if (state.context().sort_enabled)
        launch_sort_tracks(state.context(), SortKey::along_step, state.stream());
}
void step_sort_start(CoreParams const&, CoreState& state, ActionId)
{
    if (state.context().sort_enabled)
        launch_sort_tracks(state.context(), SortKey::start, state.stream());
}
void step_sort_post(CoreParams const&, CoreState& state, ActionId)
{
    if (state.context().sort_enabled)
        launch_sort_tracks(state.context(), SortKey::step_limit, state.stream());
}

}  // namespace

//---------------------------------------------------------------------------//
// Device allocations (counted)
//---------------------------------------------------------------------------//
namespace
{
std::atomic<unsigned long long> g_device_allocations{0};
}  // namespace

cudaError_t device_malloc(void** ptr, std::size_t bytes)
{
    ++g_device_allocations;
    return cudaMalloc(ptr, bytes);
}

unsigned long long device_allocation_count()
{
    return g_device_allocations.load();
}

//---------------------------------------------------------------------------//
// ActionRegistry and registration
//---------------------------------------------------------------------------//
void ActionRegistry::insert(SPConstAction action)
{
    if (!action || action->action_id() != this->next_id())
        throw std::runtime_error("action IDs must be inserted sequentially");
    labels_.emplace_back(action->label());
    actions_.push_back(std::move(action));
}

ActionId ActionRegistry::find_action(std::string_view label) const
{
    for (size_type i = 0; i < labels_.size(); ++i)
    {
        if (labels_[i] == label)
            return i;
    }
    return invalid_id;
}

void register_core_actions(ActionRegistry* reg,
                           bool uniform_field,
                           bool rz_map,
                           unsigned int track_order,
                           bool brem_combined)
{
    using O = StepActionOrder;
    auto add = [reg](std::string label,
                     std::string desc,
                     O order,
                     KernelAction::Launch launch) {
        reg->insert(std::make_shared<KernelAction>(
            reg->next_id(), std::move(label), std::move(desc), order, launch));
    };
    auto implicit = [reg](std::string label, std::string desc) {
        reg->insert(std::make_shared<ImplicitAction>(
            reg->next_id(), std::move(label), std::move(desc)));
    };
    // PhysicsParams actions
    add("pre-step", "update beginning-of-step state", O::pre, step_pre);
    implicit("msc-range", "limit range due to multiple scattering");
    implicit("eloss-range", "limit range due to energy loss");
    add("physics-discrete-select",
        "select a discrete interaction",
        O::pre_post,
        step_discrete);
    implicit("physics-integral-rejected", "reject by integral cross section");
    // Models
    add("ioni-moller-bhabha", "interact by Moller+Bhabha", O::post, step_model);
    if (brem_combined)
    {
        add("brems-combined",
            "interact by bremsstrahlung (combined SB/relativistic, e+/-)",
            O::post,
            step_model);
    }
    else
    {
        add("brems-sb", "interact by Seltzer-Berger bremsstrahlung", O::post, step_model);
        add("brems-rel",
            "interact by relativistic bremsstrahlung",
            O::post,
            step_model);
    }
    add("photoel-livermore",
        "interact by Livermore photoelectric effect",
        O::post,
        step_model);
    add("scat-klein-nishina",
        "interact by Compton scattering (simple Klein-Nishina)",
        O::post,
        step_model);
    add("conv-bethe-heitler",
        "interact by Bethe-Heitler gamma conversion",
        O::post,
        step_model);
    add("annihil-2-gamma",
        "interact by positron annihilation yielding two gammas",
        O::post,
        step_model);
    implicit("physics-failure",
             "mark a track that failed to sample an interaction");
    // The along-step action of this problem: field map, uniform field or none
    add(rz_map          ? "along-step-rzmap-msc"
        : uniform_field ? "along-step-uniform-msc"
                        : "along-step-general-linear",
        rz_map          ? "apply along-step in a R-Z map field"
        : uniform_field ? "apply along-step in a uniform field"
                        : "apply along-step for particles with no field",
        O::along,
        step_along);
    // CoreParams actions
    add("extend-from-primaries",
        "create track initializers from primaries",
        O::generate,
        step_primaries);
    add("initialize-tracks",
        "initialize track states",
        O::start,
        step_init);
    add("along-step-neutral",
        "apply along-step for neutral particles",
        O::along,
        step_along);
    implicit("geo-propagation-limit", "pause due to propagation misbehavior");
    add("geo-boundary", "cross a geometry boundary", O::post, step_boundary);
    add("tracking-cut", "kill a track and deposit its energy", O::post, step_cut);
    add("extend-from-secondaries",
        "create track initializers from secondaries",
        O::end,
        step_secondaries);
    // Optional sorting actions (SortTracksAction): step-limit sort first
    if (sorts_step_limit(track_order))
    {
        add("sort-tracks-post-step",
            "sort tracks states",
            O::sort_pre_post,
            step_sort_post);
    }
    if (sorts_along_step(track_order))
    {
        add("sort-tracks-along-step",
            "sort tracks states",
            O::sort_pre,
            step_sort_along);
    }
    if (track_order == track_order_reindex_status)
    {
        add("sort-tracks-status", "sort tracks states", O::sort_start, step_sort_start);
    }
    if (track_order == track_order_reindex_particle_type)
    {
        add("sort-tracks-start", "sort tracks states", O::sort_start, step_sort_start);
    }
    // Step gathering: the pre-step detector lookup is fused into the
    // pre-step kernel; the post-step gather applies the calorimeter tally
    add("step-gather-pre", "gather pre-step steps/hits", O::user_pre, nullptr);
    add("step-gather-post", "gather post-step steps/hits", O::user_post, step_calo);
}

//---------------------------------------------------------------------------//
// CoreParams
//---------------------------------------------------------------------------//
CoreParams::CoreParams(Input const& inp)
    : host_(build_params(inp.physics_file, inp.geometry, inp.options))
    , actions_(std::make_shared<ActionRegistry>())
{
    register_core_actions(actions_.get(),
                          host_.scalars.has_field && !host_.scalars.has_rzmap,
                          host_.scalars.has_rzmap,
                          host_.scalars.track_order,
                          host_.scalars.action_combined_brems != invalid_id);
    for (size_type i = 0; i < host_.action_labels.size(); ++i)
    {
        if (actions_->id_to_label(i) != host_.action_labels[i])
            throw std::runtime_error("action registration order mismatch");
    }

    // Pack every table into one device allocation
    Packer pk;
    HostParams const& h = host_;
    std::size_t o_reals = pk.add(h.reals);
    std::size_t o_ints = pk.add(h.ints);
    std::size_t o_part = pk.add(h.particles);
    std::size_t o_el = pk.add(h.elements);
    std::size_t o_mat = pk.add(h.materials);
    std::size_t o_fl = pk.add(h.fluct);
    std::size_t o_cut = pk.add(h.cutoffs);
    std::size_t o_grp = pk.add(h.groups);
    std::size_t o_grid = pk.add(h.grids);
    std::size_t o_lve = pk.add(h.lv_elements);
    std::size_t o_lvs = pk.add(h.lv_shells);
    std::size_t o_sb = pk.add(h.sb_tables);
    std::size_t o_rb = pk.add(h.rb_elements);
    std::size_t o_mscm = pk.add(h.msc_materials);
    std::size_t o_mscp = pk.add(h.msc_par_mat);
    std::size_t o_loop = pk.add(h.looping);
    std::size_t o_jump = pk.add(h.rng_jump);
    std::size_t o_rzmap = pk.add(h.rzmap);
    std::size_t o_rzmap_f = pk.add(h.rzmap_f);
    std::size_t o_rzdesc = pk.add(std::vector<RZMapData>(1, h.rzmap_desc));
    std::size_t o_pl = pk.add(h.surfaces);
    std::size_t o_box = pk.add(h.volumes);
    std::size_t o_no = pk.add(h.neighbor_offset);
    std::size_t o_nb = pk.add(h.neighbors);
    std::size_t o_ss = pk.add(h.sorted_surfaces);
    std::size_t o_sk = pk.add(h.sorted_key);
    std::size_t o_vm = pk.add(h.volume_material);
    std::size_t o_vd = pk.add(h.volume_detector);

    auto const& bytes = pk.bytes();
    GBX_CUDA(device_malloc(&device_storage_, bytes.size()));
    GBX_CUDA(cudaMemcpy(
        device_storage_, bytes.data(), bytes.size(), cudaMemcpyHostToDevice));
    auto* base = static_cast<unsigned char*>(device_storage_);
    device_ = h.scalars;
    device_.reals = reinterpret_cast<real_type const*>(base + o_reals);
    device_.ints = reinterpret_cast<size_type const*>(base + o_ints);
    device_.particles = reinterpret_cast<ParticleRecord const*>(base + o_part);
    device_.elements = reinterpret_cast<ElementRecord const*>(base + o_el);
    device_.materials = reinterpret_cast<MaterialRecord const*>(base + o_mat);
    device_.fluct = reinterpret_cast<UrbanFluctRecord const*>(base + o_fl);
    device_.cutoff_energy = reinterpret_cast<real_type const*>(base + o_cut);
    device_.process_groups = reinterpret_cast<ProcessGroup const*>(base + o_grp);
    device_.grids = reinterpret_cast<XsGrid const*>(base + o_grid);
    device_.livermore_elements
        = reinterpret_cast<LivermoreElement const*>(base + o_lve);
    device_.livermore_shells = reinterpret_cast<LivermoreShell const*>(base + o_lvs);
    device_.sb_tables = reinterpret_cast<SBElementTable const*>(base + o_sb);
    device_.rb_elements = reinterpret_cast<RelBremElementRecord const*>(base + o_rb);
    device_.msc.material = reinterpret_cast<UrbanMscMaterialRecord const*>(base + o_mscm);
    device_.msc.par_mat = reinterpret_cast<UrbanMscParMatRecord const*>(base + o_mscp);
    device_.looping = reinterpret_cast<LoopingRecord const*>(base + o_loop);
    device_.rng_jump = reinterpret_cast<std::uint32_t const*>(base + o_jump);
    device_.rzmap = nullptr;
    if (!h.rzmap.empty())
    {
        // The map's description, pointing at its nodes on the device
        RZMapData desc = h.rzmap_desc;
        desc.values = reinterpret_cast<FieldMapElement const*>(base + o_rzmap);
        desc.values_f = reinterpret_cast<FieldMapElementF const*>(base + o_rzmap_f);
        GBX_CUDA(cudaMemcpy(base + o_rzdesc, &desc, sizeof(desc), cudaMemcpyHostToDevice));
        device_.rzmap = reinterpret_cast<RZMapData const*>(base + o_rzdesc);
    }
    device_.geo.surfaces = reinterpret_cast<SurfaceRecord const*>(base + o_pl);
    device_.geo.volumes = reinterpret_cast<VolumeRecord const*>(base + o_box);
    device_.geo.neighbor_offset = reinterpret_cast<size_type const*>(base + o_no);
    device_.geo.neighbors = reinterpret_cast<size_type const*>(base + o_nb);
    device_.geo.sorted_surfaces = reinterpret_cast<size_type const*>(base + o_ss);
    device_.geo.sorted_key = reinterpret_cast<float const*>(base + o_sk);
    device_.geo.volume_material = reinterpret_cast<size_type const*>(base + o_vm);
    device_.geo.volume_detector = reinterpret_cast<size_type const*>(base + o_vd);
}

CoreParams::~CoreParams()
{
    if (device_storage_)
        cudaFree(device_storage_);
}

//---------------------------------------------------------------------------//
// CoreState
//---------------------------------------------------------------------------//
CoreState::CoreState(CoreParams const& params,
                     size_type num_track_slots,
                     unsigned int seed,
                     size_type initializer_capacity,
                     size_type max_events,
                     cudaStream_t stream)
    : seed_(seed), stream_(stream)
{
    if (num_track_slots == 0)
        throw std::runtime_error("number of track slots must be positive");
    size_type const n = num_track_slots;
    size_type const sec_cap = static_cast<size_type>(
        params.host().scalars.secondary_stack_factor * n);
    size_type const init_cap
        = initializer_capacity ? initializer_capacity : std::max(1u << 20, 16 * n);
    size_type const ndet = params.host().scalars.num_detectors;
    size_type const nblocks = (n + block_size - 1) / block_size;
    size_type const log_cap = 4096;
    ndet_ = ndet;

    Layout L;
    auto arr = [&L, n](std::size_t elem) { return L.reserve(elem * n); };
    std::size_t o_status = arr(1), o_track = arr(4), o_parent = arr(4),
                o_event = arr(4), o_nsteps = arr(4), o_time = arr(8),
                o_len = arr(8), o_post = arr(4), o_along = arr(4),
                o_pid = arr(4), o_energy = arr(sizeof(real_type));
    std::size_t o_pos[3], o_dir[3];
    for (int i = 0; i < 3; ++i)
        o_pos[i] = arr(8);
    for (int i = 0; i < 3; ++i)
        o_dir[i] = arr(8);
    std::size_t o_vol = arr(4), o_surf = arr(4), o_sense = arr(1),
                o_bound = arr(1), o_next = arr(8), o_nsurf = arr(4),
                o_nsense = arr(1), o_failed = arr(1), o_mat = arr(4),
                o_mfp = arr(sizeof(real_type)), o_range = arr(sizeof(real_type)),
                o_macro = arr(sizeof(real_type));
    std::size_t o_ppxs[max_processes];
    for (auto& o : o_ppxs)
        o = arr(sizeof(real_type));
    std::size_t o_edep = arr(sizeof(real_type)), o_soff = arr(4),
                o_scount = arr(4), o_elem = arr(4);
    std::size_t o_mdisp = arr(1), o_mtrue = arr(sizeof(real_type)),
                o_mgeom = arr(sizeof(real_type)), o_malpha = arr(sizeof(real_type)),
                o_mrinit = arr(sizeof(real_type)), o_mrfac = arr(sizeof(real_type)),
                o_mlmin = arr(sizeof(real_type)), o_nloop = arr(4),
                o_lekey = arr(sizeof(real_type)), o_leval = arr(sizeof(real_type)),
                o_iidx = arr(4);
    std::size_t o_rng = L.reserve(std::size_t(6) * 4 * n);
    std::size_t o_vac = arr(4), o_cnts = arr(4), o_parents = arr(4);
    std::size_t o_inits = L.reserve(sizeof(TrackInitializer) * std::size_t(init_cap));
    std::size_t o_tcount = L.reserve(4 * std::size_t(max_events));
    std::size_t o_evedep = L.reserve(8 * std::size_t(max_events));
    std::size_t o_evlive = L.reserve(4 * std::size_t(max_events));
    bool const event_tallies = params.host().scalars.event_tallies;
    std::size_t o_evdet = L.reserve(
        event_tallies ? 8 * std::size_t(max_events) * std::max<size_type>(ndet, 1) : 0);
    std::size_t o_secs = L.reserve(sizeof(Secondary) * std::size_t(sec_cap));
    std::size_t o_det = arr(4);
    std::size_t o_calo = L.reserve(8 * std::size_t(std::max<size_type>(ndet, 1)));
    size_type const prim_cap = std::max<size_type>(n, 1u << 16);
    std::size_t o_prims = L.reserve(sizeof(TrackInitializer) * std::size_t(prim_cap));
    std::size_t o_counters = L.reserve(sizeof(Counters));
    std::size_t o_bvac = L.reserve(4 * std::size_t(nblocks));
    std::size_t o_bcnt = L.reserve(4 * std::size_t(nblocks));
    std::size_t o_svac = arr(1);
    std::size_t o_scnt = arr(4);
    // Action sort: thread -> slot indirection, bin offsets, block counts
    size_type const num_actions = params.host().scalars.num_actions;
    size_type const num_materials = max_of<size_type>(1, params.host().scalars.num_materials);
    // Up to two along-step actions sorted by material take num_materials
    // bins each
    size_type const num_bins = num_actions + 2 * num_materials + 1;
    size_type const sort_blocks = (n + sort_block_size - 1) / sort_block_size;
    std::size_t o_tslots = arr(4);
    std::size_t o_aoff = L.reserve(4 * 2 * std::size_t(num_bins + 1));
    std::size_t o_shist = L.reserve(4 * std::size_t(num_bins) * sort_blocks);
    std::size_t o_work = L.reserve(sizeof(size_type));
    std::size_t o_log = L.reserve(sizeof(StepRecord) * log_cap);
    std::size_t o_stepidx = L.reserve(sizeof(size_type));

    GBX_CUDA(device_malloc(&storage_, L.size()));
    GBX_CUDA(cudaMemsetAsync(storage_, 0, L.size(), stream_));
    auto* b = static_cast<unsigned char*>(storage_);
    auto at = [b](std::size_t off) { return static_cast<void*>(b + off); };

    StateData& s = ref_;
    s.size = n;
    s.status = static_cast<std::uint8_t*>(at(o_status));
    s.track_id = static_cast<size_type*>(at(o_track));
    s.parent_id = static_cast<size_type*>(at(o_parent));
    s.event_id = static_cast<size_type*>(at(o_event));
    s.num_steps = static_cast<size_type*>(at(o_nsteps));
    s.time = static_cast<double*>(at(o_time));
    s.step_length = static_cast<double*>(at(o_len));
    s.post_step_action = static_cast<size_type*>(at(o_post));
    s.along_step_action = static_cast<size_type*>(at(o_along));
    s.particle_id = static_cast<size_type*>(at(o_pid));
    s.energy = static_cast<real_type*>(at(o_energy));
    for (int i = 0; i < 3; ++i)
    {
        s.pos[i] = static_cast<double*>(at(o_pos[i]));
        s.dir[i] = static_cast<double*>(at(o_dir[i]));
    }
    s.volume = static_cast<size_type*>(at(o_vol));
    s.surface = static_cast<size_type*>(at(o_surf));
    s.surface_sense = static_cast<std::int8_t*>(at(o_sense));
    s.boundary = static_cast<std::uint8_t*>(at(o_bound));
    s.next_step = static_cast<double*>(at(o_next));
    s.next_surface = static_cast<size_type*>(at(o_nsurf));
    s.next_sense = static_cast<std::int8_t*>(at(o_nsense));
    s.geo_failed = static_cast<std::uint8_t*>(at(o_failed));
    s.material = static_cast<size_type*>(at(o_mat));
    s.interaction_mfp = static_cast<real_type*>(at(o_mfp));
    s.dedx_range = static_cast<real_type*>(at(o_range));
    s.macro_xs = static_cast<real_type*>(at(o_macro));
    for (int i = 0; i < max_processes; ++i)
        s.per_process_xs[i] = static_cast<real_type*>(at(o_ppxs[i]));
    s.energy_deposition = static_cast<real_type*>(at(o_edep));
    s.secondaries_offset = static_cast<size_type*>(at(o_soff));
    s.secondaries_count = static_cast<size_type*>(at(o_scount));
    s.element = static_cast<size_type*>(at(o_elem));
    s.msc_displaced = static_cast<std::uint8_t*>(at(o_mdisp));
    s.msc_true_path = static_cast<real_type*>(at(o_mtrue));
    s.msc_geom_path = static_cast<real_type*>(at(o_mgeom));
    s.log_energy_key = static_cast<real_type*>(at(o_lekey));
    s.log_energy_value = static_cast<real_type*>(at(o_leval));
    s.init_indices = static_cast<size_type*>(at(o_iidx));
    s.msc_alpha = static_cast<real_type*>(at(o_malpha));
    s.msc_range_init = static_cast<real_type*>(at(o_mrinit));
    s.msc_range_factor = static_cast<real_type*>(at(o_mrfac));
    s.msc_limit_min = static_cast<real_type*>(at(o_mlmin));
    s.num_looping_steps = static_cast<size_type*>(at(o_nloop));
    auto* rng = static_cast<std::uint32_t*>(at(o_rng));
    for (int w = 0; w < 5; ++w)
        s.rng.s[w] = rng + std::size_t(w) * n;
    s.rng.weyl = rng + std::size_t(5) * n;
    s.vacancies = static_cast<size_type*>(at(o_vac));
    s.secondary_counts = static_cast<size_type*>(at(o_cnts));
    s.parents = static_cast<size_type*>(at(o_parents));
    s.initializers = static_cast<TrackInitializer*>(at(o_inits));
    s.initializer_capacity = init_cap;
    s.track_counters = static_cast<size_type*>(at(o_tcount));
    s.event_edep = static_cast<double*>(at(o_evedep));
    s.event_live = static_cast<size_type*>(at(o_evlive));
    s.event_det_edep = event_tallies ? static_cast<double*>(at(o_evdet)) : nullptr;
    s.max_events = max_events;
    s.secondaries = static_cast<Secondary*>(at(o_secs));
    s.secondary_capacity = sec_cap;
    s.detector = static_cast<size_type*>(at(o_det));
    s.calo_edep = static_cast<double*>(at(o_calo));
    s.primaries = static_cast<TrackInitializer*>(at(o_prims));
    s.primary_capacity = prim_cap;
    s.counters = static_cast<Counters*>(at(o_counters));
    s.track_slots = static_cast<size_type*>(at(o_tslots));
    s.action_offsets = static_cast<size_type*>(at(o_aoff));

    // Initial values that are not zero: fill from host staging. All-ones
    // bytes make the log(energy) keys NaN (they match no energy).
    GBX_CUDA(cudaMemsetAsync(
        s.log_energy_key, 0xFF, sizeof(real_type) * std::size_t(n), stream_));
    {
        std::vector<std::uint32_t> words;
        initialize_xorwow(seed, n, &words);
        GBX_CUDA(cudaMemcpyAsync(rng,
                                 words.data(),
                                 words.size() * 4,
                                 cudaMemcpyHostToDevice,
                                 stream_));
        std::vector<size_type> seq(n);
        for (size_type i = 0; i < n; ++i)
            seq[i] = i;
        GBX_CUDA(cudaMemcpyAsync(
            s.vacancies, seq.data(), 4 * std::size_t(n), cudaMemcpyHostToDevice, stream_));
        std::vector<size_type> inv(n, invalid_id);
        for (size_type* dst : {s.track_id,
                               s.parent_id,
                               s.event_id,
                               s.post_step_action,
                               s.along_step_action,
                               s.particle_id,
                               s.volume,
                               s.surface,
                               s.next_surface,
                               s.material,
                               s.element,
                               s.parents,
                               s.detector})
        {
            GBX_CUDA(cudaMemcpyAsync(
                dst, inv.data(), 4 * std::size_t(n), cudaMemcpyHostToDevice, stream_));
        }
        Counters c{};
        c.num_vacancies = n;
        GBX_CUDA(cudaMemcpyAsync(
            s.counters, &c, sizeof(c), cudaMemcpyHostToDevice, stream_));
        // reindex_shuffle: one random thread -> slot permutation for the
        // whole run (CoreTrackData.cc:47-56), the reference's own: a
        // Mersenne twister seeded with the number of slots shuffling the
        // identity (TrackSlotUtils.cc:21-31), visited through the first
        // offsets table's full range [offsets[0], offsets[num_bins])
        std::vector<size_type> perm;
        std::vector<size_type> offs;
        if (params.host().scalars.track_order == track_order_reindex_shuffle)
        {
            perm.resize(n);
            for (size_type i = 0; i < n; ++i)
                perm[i] = i;
            std::mt19937 gen{static_cast<unsigned int>(n)};
            std::shuffle(perm.begin(), perm.end(), gen);
            offs.assign(std::size_t(num_bins) + 1, n);
            offs[0] = 0;
            GBX_CUDA(cudaMemcpyAsync(s.track_slots,
                                     perm.data(),
                                     4 * std::size_t(n),
                                     cudaMemcpyHostToDevice,
                                     stream_));
            GBX_CUDA(cudaMemcpyAsync(s.action_offsets,
                                     offs.data(),
                                     4 * offs.size(),
                                     cudaMemcpyHostToDevice,
                                     stream_));
        }
        GBX_CUDA(cudaStreamSynchronize(stream_));
    }

    ctx_.params = params.device_ref();
    ctx_.state = s;
    ctx_.scratch.block_vacant = static_cast<size_type*>(at(o_bvac));
    ctx_.scratch.block_count = static_cast<size_type*>(at(o_bcnt));
    ctx_.scratch.vacant = static_cast<std::uint8_t*>(at(o_svac));
    ctx_.scratch.count = static_cast<size_type*>(at(o_scnt));
    ctx_.scratch.num_blocks = nblocks;
    ctx_.sort.block_hist = static_cast<size_type*>(at(o_shist));
    ctx_.sort.num_bins = num_bins;
    ctx_.sort.num_blocks = sort_blocks;
    ctx_.sort.num_actions = num_actions;
    ctx_.sort.num_materials = num_materials;
    ctx_.sort.material_actions[0] = invalid_id;
    ctx_.sort.material_actions[1] = invalid_id;
    ctx_.sort.track_order = params.host().scalars.track_order;
    ctx_.work_counter = static_cast<size_type*>(at(o_work));
    // Persistent charged along-step: on by default in the mixed-precision
    // build, where it outruns the one-thread-per-track kernel; in FP64 the
    // diverged FP64 multiple-scattering code makes it slower
    ctx_.along_block_size = block_size;
    ctx_.sort_enabled = true;
    ctx_.partition_slots = false;
    {
        int device = 0, sms = 0;
        GBX_CUDA(cudaGetDevice(&device));
        GBX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        ctx_.range_blocks = std::min<unsigned int>(
            (n + block_size - 1) / block_size, 8u * static_cast<unsigned int>(sms));
    }
    ctx_.persistent_blocks = sizeof(real_type) < sizeof(double)
                                 ? persistent_along_blocks(ctx_.along_block_size)
                                 : 0;
    ctx_.log = static_cast<StepRecord*>(at(o_log));
    ctx_.log_capacity = log_cap;
    ctx_.step_index = static_cast<size_type*>(at(o_stepidx));

    pinned_capacity_ = prim_cap;
    GBX_CUDA(cudaMallocHost(&pinned_primaries_,
                            sizeof(TrackInitializer) * std::size_t(prim_cap)));
}

CoreState::~CoreState()
{
    if (hits_storage_)
        cudaFree(hits_storage_);
    if (storage_)
        cudaFree(storage_);
    if (pinned_primaries_)
        cudaFreeHost(pinned_primaries_);
}

void CoreState::set_step_output(unsigned int selection,
                                bool nonzero_energy_deposition,
                                size_type capacity)
{
    if (selection & ~unsigned(step_select_all))
        throw std::runtime_error("unknown step output selection bits");
    GBX_CUDA(cudaStreamSynchronize(stream_));
    if (hits_storage_)
    {
        GBX_CUDA(cudaFree(hits_storage_));
        hits_storage_ = nullptr;
    }
    ref_.pre_time = ref_.pre_pos = ref_.pre_dir = ref_.pre_energy = nullptr;
    ctx_.hits = StepHitsRef{};
    ctx_.hit_block_offsets = nullptr;
    // Start from an empty output without a pending overflow
    Counters c = this->counters();
    c.num_hits = 0;
    c.error_flags &= ~size_type(error_hit_overflow);
    GBX_CUDA(cudaMemcpyAsync(
        ref_.counters, &c, sizeof(c), cudaMemcpyHostToDevice, stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    if (capacity == 0)
    {
        ctx_.state = ref_;
        return;
    }

    // One allocation: pre-step points per slot, records, block offsets
    std::size_t const n = ref_.size;
    std::size_t const cap = capacity;
    size_type const nblocks = (ref_.size + block_size - 1) / block_size;
    Layout L;
    auto slot_array = [&](unsigned int bit, std::size_t per_slot) {
        return (selection & bit) ? L.reserve(per_slot * n) : std::size_t(-1);
    };
    auto hit_array = [&](unsigned int bit, std::size_t per_hit) {
        return (bit == 0 || (selection & bit)) ? L.reserve(per_hit * cap)
                                               : std::size_t(-1);
    };
    std::size_t const o_ptime = slot_array(step_pre_time, 8);
    std::size_t const o_ppos = slot_array(step_pre_pos, 24);
    std::size_t const o_pdir = slot_array(step_pre_dir, 24);
    std::size_t const o_pen = slot_array(step_pre_energy, 8);
    std::size_t const o_step = hit_array(0, 4), o_det = hit_array(0, 4),
                      o_track = hit_array(0, 4);
    std::size_t const o_event = hit_array(step_event_id, 4),
                      o_parent = hit_array(step_parent_id, 4),
                      o_count = hit_array(step_track_step_count, 4),
                      o_particle = hit_array(step_particle, 4),
                      o_len = hit_array(step_step_length, 8),
                      o_edep = hit_array(step_energy_deposition, 8),
                      o_htime = hit_array(step_pre_time, 8),
                      o_hpos = hit_array(step_pre_pos, 24),
                      o_hdir = hit_array(step_pre_dir, 24),
                      o_hen = hit_array(step_pre_energy, 8),
                      o_qtime = hit_array(step_post_time, 8),
                      o_qpos = hit_array(step_post_pos, 24),
                      o_qdir = hit_array(step_post_dir, 24),
                      o_qen = hit_array(step_post_energy, 8);
    std::size_t const o_blocks = L.reserve(4 * std::size_t(nblocks));
    GBX_CUDA(device_malloc(&hits_storage_, L.size()));
    GBX_CUDA(cudaMemsetAsync(hits_storage_, 0, L.size(), stream_));
    auto* b = static_cast<unsigned char*>(hits_storage_);
    auto at = [b](std::size_t off) -> void* {
        return off == std::size_t(-1) ? nullptr : static_cast<void*>(b + off);
    };
    ref_.pre_time = static_cast<double*>(at(o_ptime));
    ref_.pre_pos = static_cast<double*>(at(o_ppos));
    ref_.pre_dir = static_cast<double*>(at(o_pdir));
    ref_.pre_energy = static_cast<double*>(at(o_pen));
    StepHitsRef& h = ctx_.hits;
    h.capacity = capacity;
    h.selection = selection;
    h.nonzero_energy_deposition = nonzero_energy_deposition;
    h.step = static_cast<size_type*>(at(o_step));
    h.detector = static_cast<size_type*>(at(o_det));
    h.track_id = static_cast<size_type*>(at(o_track));
    h.event_id = static_cast<size_type*>(at(o_event));
    h.parent_id = static_cast<size_type*>(at(o_parent));
    h.track_step_count = static_cast<size_type*>(at(o_count));
    h.particle = static_cast<size_type*>(at(o_particle));
    h.step_length = static_cast<double*>(at(o_len));
    h.energy_deposition = static_cast<double*>(at(o_edep));
    h.pre_time = static_cast<double*>(at(o_htime));
    h.pre_pos = static_cast<double*>(at(o_hpos));
    h.pre_dir = static_cast<double*>(at(o_hdir));
    h.pre_energy = static_cast<double*>(at(o_hen));
    h.post_time = static_cast<double*>(at(o_qtime));
    h.post_pos = static_cast<double*>(at(o_qpos));
    h.post_dir = static_cast<double*>(at(o_qdir));
    h.post_energy = static_cast<double*>(at(o_qen));
    ctx_.hit_block_offsets = static_cast<size_type*>(at(o_blocks));
    ctx_.state = ref_;
    GBX_CUDA(cudaStreamSynchronize(stream_));
}

size_type CoreState::read_step_output(StepHitsRef const& out)
{
    StepHitsRef const& h = ctx_.hits;
    if (!h.enabled())
        throw std::runtime_error("step output is not enabled");
    Counters c = this->counters();
    if (c.error_flags & error_hit_overflow)
    {
        size_type const held = c.num_hits;
        c.num_hits = 0;
        c.error_flags &= ~size_type(error_hit_overflow);
        GBX_CUDA(cudaMemcpyAsync(
            ref_.counters, &c, sizeof(c), cudaMemcpyHostToDevice, stream_));
        GBX_CUDA(cudaStreamSynchronize(stream_));
        throw std::runtime_error(
            "step output overflowed its capacity of " + std::to_string(h.capacity)
            + " records (" + std::to_string(held)
            + " held): hits of later steps were dropped; read the output more "
              "often or raise its capacity");
    }
    size_type const n = c.num_hits;
    if (n > out.capacity)
        throw std::runtime_error("step output holds " + std::to_string(n)
                                 + " records, more than the "
                                 + std::to_string(out.capacity)
                                 + " the destination arrays hold");
    auto copy = [&](void* dst, void const* src, std::size_t per_hit) {
        if (dst && src && n > 0)
        {
            GBX_CUDA(cudaMemcpyAsync(
                dst, src, per_hit * n, cudaMemcpyDeviceToHost, stream_));
        }
    };
    copy(out.step, h.step, 4);
    copy(out.detector, h.detector, 4);
    copy(out.track_id, h.track_id, 4);
    copy(out.event_id, h.event_id, 4);
    copy(out.parent_id, h.parent_id, 4);
    copy(out.track_step_count, h.track_step_count, 4);
    copy(out.particle, h.particle, 4);
    copy(out.step_length, h.step_length, 8);
    copy(out.energy_deposition, h.energy_deposition, 8);
    copy(out.pre_time, h.pre_time, 8);
    copy(out.pre_pos, h.pre_pos, 24);
    copy(out.pre_dir, h.pre_dir, 24);
    copy(out.pre_energy, h.pre_energy, 8);
    copy(out.post_time, h.post_time, 8);
    copy(out.post_pos, h.post_pos, 24);
    copy(out.post_dir, h.post_dir, 24);
    copy(out.post_energy, h.post_energy, 8);
    GBX_CUDA(cudaMemsetAsync(
        &ref_.counters->num_hits, 0, sizeof(size_type), stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    return n;
}

void CoreState::generate_primaries(PrimaryGeneratorData gen)
{
    if (pending_primaries_ != 0)
        throw std::runtime_error("multiple consecutive primary insertions");
    std::size_t const n = std::size_t(gen.num_events) * gen.primaries_per_event;
    if (n == 0)
        return;
    if (n > pinned_capacity_)
        throw std::runtime_error("too many primaries for one insertion");
    if (std::size_t(gen.first_event) + gen.num_events > ref_.max_events)
        throw std::runtime_error("generated event IDs exceed the stepper's event capacity "
                                 + std::to_string(ref_.max_events));
    for (size_type e = 0; e < gen.num_events; ++e)
    {
        if (primaries_per_event_.count(gen.first_event + e))
            throw std::runtime_error("event " + std::to_string(gen.first_event + e)
                                     + " already has primaries");
    }
    for (size_type e = 0; e < gen.num_events; ++e)
        primaries_per_event_[gen.first_event + e] = gen.primaries_per_event;
    gen.stepper_seed = seed_;
    GBX_CUDA(cudaStreamSynchronize(stream_));
    launch_generate_primaries(ctx_, gen, stream_);
    GBX_CUDA(cudaGetLastError());
    pending_primaries_ = static_cast<size_type>(n);
}

void CoreState::insert_primaries(TrackInitializer const* host_primaries, size_type n)
{
    if (pending_primaries_ != 0)
        throw std::runtime_error("multiple consecutive primary insertions");
    if (n > pinned_capacity_)
        throw std::runtime_error("too many primaries for one insertion");
    if (n == 0)
        return;
    // Stage through pinned memory so the copy is asynchronous
    GBX_CUDA(cudaStreamSynchronize(stream_));
    std::memcpy(pinned_primaries_, host_primaries, sizeof(TrackInitializer) * n);
    for (size_type i = 0; i < n; ++i)
    {
        TrackInitializer& ti = pinned_primaries_[i];
        if (ti.event_id >= ref_.max_events)
            throw std::runtime_error("primary event ID " + std::to_string(ti.event_id)
                                     + " exceeds the stepper's event capacity "
                                     + std::to_string(ref_.max_events));
        // Seed of a per-track random stream: the stepper seed, the event
        // and the primary's index among that event's primaries
        size_type const index = primaries_per_event_[ti.event_id]++;
        SplitMix64 sm{(std::uint64_t(seed_) << 32) | ti.event_id};
        SplitMix64 sm2{sm() + 0x9e3779b97f4a7c15ull * (std::uint64_t(index) + 1)};
        ti.rng_key = sm2();
    }
    GBX_CUDA(cudaMemcpyAsync(ref_.primaries,
                             pinned_primaries_,
                             sizeof(TrackInitializer) * n,
                             cudaMemcpyHostToDevice,
                             stream_));
    pending_primaries_ = n;
}

void CoreState::set_tuning(std::string const& name, long long value)
{
    if (name == "along_block_size")
    {
        if (value != 64 && value != 128 && value != 256 && value != 512)
        {
            throw std::runtime_error("along_block_size must be 64, 128, 256 or 512");
        }
        ctx_.along_block_size = static_cast<int>(value);
        if (ctx_.persistent_blocks > 0)
            ctx_.persistent_blocks = persistent_along_blocks(ctx_.along_block_size);
    }
    else if (name == "along_persistent")
    {
        ctx_.persistent_blocks
            = value ? persistent_along_blocks(ctx_.along_block_size) : 0;
        if (value && ctx_.persistent_blocks == 0)
            throw std::runtime_error("persistent along-step kernel cannot be resident");
    }
    else if (name == "sort")
    {
        ctx_.sort_enabled = value != 0;
    }
    else if (name == "sort_material")
    {
        // Bit 0: the charged along-step action, bit 1: the neutral one
        if (value < 0 || value > 3)
            throw std::runtime_error("sort_material must be 0-3");
        size_type ids[2];
        int n = 0;
        size_type const charged = ctx_.params.action_along_step;
        size_type const neutral = ctx_.params.action_along_step_neutral;
        if ((value & 1) && charged != invalid_id)
            ids[n++] = charged;
        if ((value & 2) && neutral != invalid_id)
            ids[n++] = neutral;
        if (n == 2 && ids[1] < ids[0])
            std::swap(ids[0], ids[1]);
        ctx_.sort.material_actions[0] = n > 0 ? ids[0] : invalid_id;
        ctx_.sort.material_actions[1] = n > 1 ? ids[1] : invalid_id;
        sort_material_ = static_cast<int>(value);
    }
    else if (name == "partition_slots")
    {
        if (value && !ctx_.params.rng_per_track)
        {
            throw std::runtime_error(
                "partition_slots needs per-track random streams (rng_per_track)");
        }
        ctx_.partition_slots = value != 0;
    }
    else
    {
        throw std::runtime_error("unknown tuning parameter '" + name + "'");
    }
}

long long CoreState::tuning(std::string const& name) const
{
    if (name == "along_block_size")
        return ctx_.along_block_size;
    if (name == "along_persistent")
        return ctx_.persistent_blocks > 0;
    if (name == "sort")
        return ctx_.sort_enabled;
    if (name == "partition_slots")
        return ctx_.partition_slots;
    if (name == "sort_material")
        return sort_material_;
    throw std::runtime_error("unknown tuning parameter '" + name + "'");
}

void CoreState::reseed(unsigned long long event_id)
{
    launch_reseed(ctx_, seed_, event_id, stream_);
    GBX_CUDA(cudaGetLastError());
    // TrackInitParams::reset_track_ids: every per-event counter restarts
    GBX_CUDA(cudaMemsetAsync(
        ref_.track_counters, 0, sizeof(size_type) * ref_.max_events, stream_));
}

std::vector<size_type> CoreState::sorted_action_sizes(int key) const
{
    SortScratch const& srt = ctx_.sort;
    std::size_t const table = std::size_t(srt.num_bins) + 1;
    std::vector<size_type> off(table);
    GBX_CUDA(cudaMemcpyAsync(off.data(),
                             ref_.action_offsets + (key ? table : 0),
                             sizeof(size_type) * table,
                             cudaMemcpyDeviceToHost,
                             stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    std::vector<size_type> out(srt.num_actions);
    unsigned int const order = ctx_.params.track_order;
    if (!(key == 0 ? sorts_along_step(order) : sorts_step_limit(order)))
        return std::vector<size_type>(srt.num_actions, 0);
    for (size_type a = 0; a < srt.num_actions; ++a)
    {
        size_type first = a;
        size_type end = a + 1;
        if (key == 0)
            along_bins(srt, a, &first, &end);
        out[a] = off[end] - off[first];
    }
    return out;
}

std::vector<size_type> CoreState::event_live(size_type n) const
{
    if (n > ref_.max_events)
        throw std::runtime_error("more events requested than the stepper holds");
    std::vector<size_type> out(n);
    if (n == 0)
        return out;
    launch_count_event_live(ctx_, n, stream_);
    GBX_CUDA(cudaGetLastError());
    GBX_CUDA(cudaMemcpyAsync(out.data(),
                             ref_.event_live,
                             sizeof(size_type) * n,
                             cudaMemcpyDeviceToHost,
                             stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    return out;
}

std::vector<double> CoreState::event_energy_deposition(size_type n, bool clear)
{
    if (n > ref_.max_events)
        throw std::runtime_error("more events requested than the stepper holds");
    std::vector<double> out(n);
    if (n == 0)
        return out;
    GBX_CUDA(cudaMemcpyAsync(out.data(),
                             ref_.event_edep,
                             sizeof(double) * n,
                             cudaMemcpyDeviceToHost,
                             stream_));
    if (clear)
    {
        GBX_CUDA(cudaMemsetAsync(ref_.event_edep, 0, sizeof(double) * n, stream_));
    }
    GBX_CUDA(cudaStreamSynchronize(stream_));
    return out;
}

std::vector<double>
CoreState::event_detector_energy_deposition(size_type first, size_type n, bool clear)
{
    if (!ref_.event_det_edep)
        throw std::runtime_error("per-event tallies are not enabled");
    if (std::size_t(first) + n > ref_.max_events)
        throw std::runtime_error("more events requested than the stepper holds");
    std::size_t const ndet = ndet_;
    std::vector<double> out(std::size_t(n) * ndet);
    if (out.empty())
        return out;
    double* src = ref_.event_det_edep + std::size_t(first) * ndet;
    GBX_CUDA(cudaMemcpyAsync(
        out.data(), src, sizeof(double) * out.size(), cudaMemcpyDeviceToHost, stream_));
    if (clear)
    {
        GBX_CUDA(cudaMemsetAsync(src, 0, sizeof(double) * out.size(), stream_));
    }
    GBX_CUDA(cudaStreamSynchronize(stream_));
    return out;
}

Counters CoreState::counters() const
{
    Counters c;
    GBX_CUDA(cudaMemcpyAsync(
        &c, ref_.counters, sizeof(c), cudaMemcpyDeviceToHost, stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    return c;
}

size_type CoreState::step_index() const
{
    size_type idx;
    GBX_CUDA(cudaMemcpyAsync(
        &idx, ctx_.step_index, sizeof(idx), cudaMemcpyDeviceToHost, stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    return idx;
}

std::vector<StepRecord> CoreState::step_log(size_type first, size_type n) const
{
    std::vector<StepRecord> all(ctx_.log_capacity);
    GBX_CUDA(cudaMemcpyAsync(all.data(),
                             ctx_.log,
                             sizeof(StepRecord) * all.size(),
                             cudaMemcpyDeviceToHost,
                             stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    std::vector<StepRecord> result(n);
    for (size_type i = 0; i < n; ++i)
        result[i] = all[(first + i) % ctx_.log_capacity];
    return result;
}

//---------------------------------------------------------------------------//
// ActionSequence
//---------------------------------------------------------------------------//
ActionSequence::ActionSequence(ActionRegistry const& reg)
{
    for (size_type i = 0; i < reg.num_actions(); ++i)
    {
        if (auto const* sa = dynamic_cast<CoreStepActionInterface const*>(
                reg.action(i).get()))
        {
            actions_.push_back(sa);
        }
    }
    // Sort by (order, ID)
    std::stable_sort(actions_.begin(),
                     actions_.end(),
                     [](CoreStepActionInterface const* a,
                        CoreStepActionInterface const* b) {
                         if (a->order() != b->order())
                             return a->order() < b->order();
                         return a->action_id() < b->action_id();
                     });
    num_ids_ = reg.num_actions();
    elapsed_.assign(num_ids_, 0.0);
    launches_.assign(num_ids_, 0);
    pending_.assign(num_ids_, false);
}

ActionSequence::~ActionSequence()
{
    for (auto e : start_)
        cudaEventDestroy(e);
    for (auto e : stop_)
        cudaEventDestroy(e);
}

void ActionSequence::enable_action_times(bool enable)
{
    if (enable && start_.empty())
    {
        start_.resize(num_ids_);
        stop_.resize(num_ids_);
        for (size_type i = 0; i < num_ids_; ++i)
        {
            GBX_CUDA(cudaEventCreate(&start_[i]));
            GBX_CUDA(cudaEventCreate(&stop_[i]));
        }
    }
    timing_ = enable;
}

void ActionSequence::collect() const
{
    for (size_type i = 0; i < num_ids_; ++i)
    {
        if (pending_[i])
        {
            float ms = 0;
            GBX_CUDA(cudaEventSynchronize(stop_[i]));
            GBX_CUDA(cudaEventElapsedTime(&ms, start_[i], stop_[i]));
            elapsed_[i] += ms;
            pending_[i] = false;
        }
    }
}

std::vector<double> ActionSequence::action_times() const
{
    this->collect();
    return elapsed_;
}

void ActionSequence::reset_action_times()
{
    this->collect();
    elapsed_.assign(num_ids_, 0.0);
    launches_.assign(num_ids_, 0);
}

void ActionSequence::step(CoreParams const& params, CoreState& state) const
{
    if (!timing_)
    {
        for (auto const* a : actions_)
            a->step(params, state);
        return;
    }
    // Events bracket each action on the state's stream; accumulate the
    // previous step's timings before reusing the events
    this->collect();
    for (auto const* a : actions_)
    {
        ActionId id = a->action_id();
        GBX_CUDA(cudaEventRecord(start_[id], state.stream()));
        a->step(params, state);
        GBX_CUDA(cudaEventRecord(stop_[id], state.stream()));
        pending_[id] = true;
        ++launches_[id];
    }
}

//---------------------------------------------------------------------------//
// Stepper
//---------------------------------------------------------------------------//
Stepper::Stepper(StepperInput const& input)
    : params_(input.params), use_graph_(input.use_graph)
{
    if (!params_)
        throw std::runtime_error("stepper requires params");
    GBX_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    state_ = std::make_unique<CoreState>(*params_,
                                         input.num_track_slots,
                                         input.seed,
                                         input.initializer_capacity,
                                         input.max_events,
                                         stream_);
    actions_ = std::make_unique<ActionSequence>(params_->action_reg());
}

Stepper::~Stepper()
{
    this->clear_graphs();
    state_.reset();
    if (stream_)
        cudaStreamDestroy(stream_);
}

void Stepper::clear_graphs()
{
    for (int i = 0; i < 2; ++i)
    {
        if (graph_exec_[i])
            cudaGraphExecDestroy(graph_exec_[i]);
        if (graph_[i])
            cudaGraphDestroy(graph_[i]);
        graph_exec_[i] = nullptr;
        graph_[i] = nullptr;
    }
}

void Stepper::build_graph()
{
    int const k = state_->context().sort_enabled ? 1 : 0;
    GBX_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    actions_->step(*params_, *state_);
    GBX_CUDA(cudaStreamEndCapture(stream_, &graph_[k]));
    GBX_CUDA(cudaGraphInstantiate(&graph_exec_[k], graph_[k], 0));
}

void Stepper::update_sort_policy()
{
    if (sort_threshold_ <= 0)
        return;
    bool const sort = static_cast<long long>(last_active_) >= sort_threshold_;
    if (sort != state_->context().sort_enabled)
        state_->set_tuning("sort", sort);
}

void Stepper::set_step_output(unsigned int selection,
                              bool nonzero_energy_deposition,
                              size_type capacity)
{
    state_->set_step_output(selection, nonzero_energy_deposition, capacity);
    this->clear_graphs();
}

void Stepper::set_tuning(std::string const& name, long long value)
{
    if (name == "sort_threshold")
    {
        if (value < 0)
            throw std::runtime_error("sort_threshold must be nonnegative");
        sort_threshold_ = value;
        if (value == 0)
            state_->set_tuning("sort", 1);
    }
    else
    {
        state_->set_tuning(name, value);
    }
    this->clear_graphs();
}

long long Stepper::tuning(std::string const& name) const
{
    if (name == "sort_threshold")
        return sort_threshold_;
    return state_->tuning(name);
}

size_type Stepper::graph_kernel_count()
{
    int const k = state_->context().sort_enabled ? 1 : 0;
    if (!graph_exec_[k])
        this->build_graph();
    std::size_t num_nodes = 0;
    GBX_CUDA(cudaGraphGetNodes(graph_[k], nullptr, &num_nodes));
    std::vector<cudaGraphNode_t> nodes(num_nodes);
    GBX_CUDA(cudaGraphGetNodes(graph_[k], nodes.data(), &num_nodes));
    size_type kernels = 0;
    for (auto node : nodes)
    {
        cudaGraphNodeType type;
        GBX_CUDA(cudaGraphNodeGetType(node, &type));
        if (type == cudaGraphNodeTypeKernel)
            ++kernels;
    }
    return kernels;
}

void Stepper::launch_steps(size_type count)
{
    for (size_type i = 0; i < count; ++i)
    {
        if (use_graph_ && state_->pending_primaries() == 0
            && !actions_->action_times_enabled())
        {
            int const k = state_->context().sort_enabled ? 1 : 0;
            if (!graph_exec_[k])
                this->build_graph();
            GBX_CUDA(cudaGraphLaunch(graph_exec_[k], stream_));
        }
        else
        {
            actions_->step(*params_, *state_);
        }
    }
    GBX_CUDA(cudaGetLastError());
}

StepperResult Stepper::read_record(size_type index) const
{
    StepRecord r = state_->step_log(index, 1).front();
    StepperResult out;
    out.generated = r.generated;
    out.queued = r.queued;
    out.active = r.active;
    out.alive = r.alive;
    return out;
}

StepperResult Stepper::operator()(std::vector<TrackInitializer> const& primaries)
{
    state_->insert_primaries(primaries.data(),
                             static_cast<size_type>(primaries.size()));
    return (*this)();
}

StepperResult Stepper::operator()()
{
    this->update_sort_policy();
    size_type idx = state_->step_index();
    this->launch_steps(1);
    Counters c = state_->counters();
    if (c.error_flags & error_initializer_overflow)
        throw std::runtime_error("insufficient capacity for track initializers");
    StepperResult r = this->read_record(idx);
    last_active_ = r.alive + r.queued;
    return r;
}

std::vector<StepperResult> Stepper::run_until_empty(size_type max_steps,
                                                    size_type batch)
{
    std::vector<StepperResult> results;
    size_type first = state_->step_index();
    batch = std::max<size_type>(1, std::min(batch, state_->log_capacity()));
    size_type taken = 0;
    bool done = false;
    while (!done && taken < max_steps)
    {
        size_type n = std::min(batch, max_steps - taken);
        this->update_sort_policy();
        this->launch_steps(n);
        Counters c = state_->counters();
        if (c.error_flags & error_initializer_overflow)
            throw std::runtime_error("insufficient capacity for track initializers");
        auto recs = state_->step_log(first + taken, n);
        for (auto const& r : recs)
        {
            StepperResult out;
            out.generated = r.generated;
            out.queued = r.queued;
            out.active = r.active;
            out.alive = r.alive;
            results.push_back(out);
            last_active_ = out.alive + out.queued;
            if (!out)
            {
                done = true;
                break;
            }
        }
        taken += n;
    }
    return results;
}

void Stepper::warm_up()
{
    Counters c = state_->counters();
    if (c.num_active != 0 || c.num_initializers != 0 || state_->pending_primaries() != 0)
        throw std::runtime_error("cannot warm up when state has active tracks");
    // Both sort states when the sort threshold switches between them
    bool const sorted = state_->context().sort_enabled;
    auto one_step = [this] {
        if (use_graph_ && !actions_->action_times_enabled())
        {
            int const k = state_->context().sort_enabled ? 1 : 0;
            if (!graph_exec_[k])
                this->build_graph();
            GBX_CUDA(cudaGraphLaunch(graph_exec_[k], stream_));
        }
        else
        {
            actions_->step(*params_, *state_);
        }
    };
    one_step();
    if (sort_threshold_ > 0 && params_->host().scalars.track_order != 0)
    {
        state_->set_tuning("sort", !sorted);
        one_step();
        state_->set_tuning("sort", sorted);
    }
    GBX_CUDA(cudaStreamSynchronize(stream_));
    c = state_->counters();
    if (c.num_active != 0 || c.num_initializers != 0)
        throw std::runtime_error("warm-up step left tracks in the state");
}

void Stepper::reseed(unsigned long long event_id)
{
    state_->reseed(event_id);
    GBX_CUDA(cudaStreamSynchronize(stream_));
}

void Stepper::kill_active()
{
    launch_kill_active(state_->context(), stream_);
    GBX_CUDA(cudaStreamSynchronize(stream_));
}

std::vector<double> Stepper::energy_deposition() const
{
    std::vector<double> result(params_->host().scalars.num_detectors);
    GBX_CUDA(cudaMemcpyAsync(result.data(),
                             state_->ref().calo_edep,
                             sizeof(double) * result.size(),
                             cudaMemcpyDeviceToHost,
                             stream_));
    GBX_CUDA(cudaStreamSynchronize(stream_));
    return result;
}

void Stepper::clear_energy_deposition()
{
    GBX_CUDA(cudaMemsetAsync(state_->ref().calo_edep,
                             0,
                             sizeof(double) * params_->host().scalars.num_detectors,
                             stream_));
}

}  // namespace gbx
