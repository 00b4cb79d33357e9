// Implementation of the C ABI declared in include/celeritas_gb300.h.
#include "../../include/celeritas_gb300.h"

#include <algorithm>
#include <cstring>
#include <exception>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "gbx/Libm.hh"
#include "host/Core.hh"

struct gbx_params_s
{
    std::shared_ptr<gbx::CoreParams const> params;
    unsigned int initializer_capacity{0};  //!< Queue of each stepper (0: default)
};

struct gbx_stepper_s
{
    std::unique_ptr<gbx::Stepper> stepper;
    int device{-1};  //!< Device current when the stepper was created
};

namespace
{
thread_local std::string g_last_error;

//! y[i] = f(x[i]) with the stepping loop's FP64 elementary functions
__global__ void libm_evaluate_kernel(int function, double const* x, double* y, size_t n)
{
    namespace L = gbx::libm;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
    {
        double const v = x[i];
        double r;
        switch (function)
        {
            case GBX_LIBM_EXP: r = L::exp(v); break;
            case GBX_LIBM_LOG: r = L::log(v); break;
            case GBX_LIBM_SIN: r = L::sin(v); break;
            case GBX_LIBM_COS: r = L::cos(v); break;
            case GBX_LIBM_TANH: r = L::tanh(v); break;
            case GBX_LIBM_LOG1P: r = L::log1p(v); break;
            case GBX_LIBM_EXPM1: r = L::expm1(v); break;
            default: r = L::cbrt(v); break;
        }
        y[i] = r;
    }
}

template<class F>
int guarded(F&& f)
{
    try
    {
        f();
        g_last_error.clear();
        return 0;
    }
    catch (std::exception const& e)
    {
        g_last_error = e.what();
    }
    catch (...)
    {
        g_last_error = "unknown error";
    }
    return 1;
}

int copy_label(std::string const& s, char* buf, size_t buf_size)
{
    if (!buf || buf_size == 0)
        return 1;
    std::size_t n = std::min(s.size(), buf_size - 1);
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
    return 0;
}

std::vector<gbx::TrackInitializer>
to_initializers(gbx::ParamsData const& p, gbx_primary const* prim, size_t n)
{
    std::vector<gbx::TrackInitializer> result(n);
    for (size_t i = 0; i < n; ++i)
    {
        gbx::TrackInitializer& ti = result[i];
        ti = {};
        if (prim[i].pdg == 11)
            ti.particle_id = p.electron_id;
        else if (prim[i].pdg == -11)
            ti.particle_id = p.positron_id;
        else if (prim[i].pdg == 22)
            ti.particle_id = p.gamma_id;
        else
            throw std::runtime_error("unsupported primary PDG "
                                     + std::to_string(prim[i].pdg));
        ti.energy = prim[i].energy;
        ti.pos = {prim[i].pos[0], prim[i].pos[1], prim[i].pos[2]};
        ti.dir = {prim[i].dir[0], prim[i].dir[1], prim[i].dir[2]};
        ti.time = prim[i].time;
        ti.event_id = prim[i].event_id;
        ti.track_id = gbx::invalid_id;
        ti.parent_id = gbx::invalid_id;
    }
    return result;
}

gbx_step_result to_c(gbx::StepperResult const& r)
{
    return {r.generated, r.queued, r.active, r.alive};
}

//! Address and size of a named state array
struct FieldRef
{
    void* ptr{nullptr};
    std::size_t elem{0};
    std::size_t count{0};
};

FieldRef find_field(gbx::CoreState& st, std::string const& name)
{
    using namespace gbx;
    StateData const& s = st.ref();
    std::size_t n = s.size;
    auto f = [n](auto* p) {
        return FieldRef{
            static_cast<void*>(p), sizeof(std::remove_pointer_t<decltype(p)>), n};
    };
    if (name == "status") return f(s.status);
    if (name == "track_id") return f(s.track_id);
    if (name == "parent_id") return f(s.parent_id);
    if (name == "event_id") return f(s.event_id);
    if (name == "num_steps") return f(s.num_steps);
    if (name == "time") return f(s.time);
    if (name == "step_length") return f(s.step_length);
    if (name == "post_step_action") return f(s.post_step_action);
    if (name == "along_step_action") return f(s.along_step_action);
    if (name == "particle_id") return f(s.particle_id);
    if (name == "energy") return f(s.energy);
    if (name == "pos_x") return f(s.pos[0]);
    if (name == "pos_y") return f(s.pos[1]);
    if (name == "pos_z") return f(s.pos[2]);
    if (name == "dir_x") return f(s.dir[0]);
    if (name == "dir_y") return f(s.dir[1]);
    if (name == "dir_z") return f(s.dir[2]);
    if (name == "volume") return f(s.volume);
    if (name == "surface") return f(s.surface);
    if (name == "surface_sense") return f(s.surface_sense);
    if (name == "boundary") return f(s.boundary);
    if (name == "next_step") return f(s.next_step);
    if (name == "next_surface") return f(s.next_surface);
    if (name == "next_sense") return f(s.next_sense);
    if (name == "geo_failed") return f(s.geo_failed);
    if (name == "num_looping_steps") return f(s.num_looping_steps);
    if (name == "material") return f(s.material);
    if (name == "interaction_mfp") return f(s.interaction_mfp);
    if (name == "dedx_range") return f(s.dedx_range);
    if (name == "macro_xs") return f(s.macro_xs);
    for (int i = 0; i < max_processes; ++i)
    {
        if (name == "per_process_xs_" + std::to_string(i))
            return f(s.per_process_xs[i]);
    }
    if (name == "energy_deposition") return f(s.energy_deposition);
    if (name == "secondaries_offset") return f(s.secondaries_offset);
    if (name == "secondaries_count") return f(s.secondaries_count);
    if (name == "element") return f(s.element);
    if (name == "detector") return f(s.detector);
    if (name == "vacancies") return f(s.vacancies);
    if (name == "parents") return f(s.parents);
    if (name == "secondary_counts") return f(s.secondary_counts);
    if (name == "rng")
        return FieldRef{s.rng.s[0], sizeof(std::uint32_t), 6 * n};
    if (name == "track_slots") return f(s.track_slots);
    if (name == "action_offsets")
        return FieldRef{s.action_offsets,
                        sizeof(size_type),
                        2 * std::size_t(st.context().sort.num_bins + 1)};
    if (name == "counters")
        return FieldRef{s.counters, sizeof(Counters), 1};
    if (name == "primaries")
        return FieldRef{s.primaries, sizeof(TrackInitializer), s.primary_capacity};
    if (name == "initializers")
        return FieldRef{s.initializers, sizeof(TrackInitializer), s.initializer_capacity};
    if (name == "secondaries")
        return FieldRef{s.secondaries, sizeof(Secondary), s.secondary_capacity};
    if (name == "track_counters")
        return FieldRef{s.track_counters, sizeof(size_type), s.max_events};
    throw std::runtime_error("unknown state field '" + name + "'");
}

gbx::GeometrySpec geometry_by_name(std::string const& name)
{
    return gbx::make_geometry(name);
}

}  // namespace

extern "C" {

const char* gbx_last_error(void)
{
    return g_last_error.c_str();
}

void gbx_field_driver_options_default(gbx_field_driver_options* options)
{
    if (!options)
        return;
    gbx::FieldOptions const o;
    options->minimum_step = o.minimum_step;
    options->delta_chord = o.delta_chord;
    options->delta_intersection = o.delta_intersection;
    options->epsilon_step = o.epsilon_step;
    options->epsilon_rel_max = o.epsilon_rel_max;
    options->errcon = o.errcon;
    options->pgrow = o.pgrow;
    options->pshrink = o.pshrink;
    options->safety = o.safety;
    options->max_stepping_increase = o.max_stepping_increase;
    options->max_stepping_decrease = o.max_stepping_decrease;
    options->max_nsteps = o.max_nsteps;
    options->max_substeps = o.max_substeps;
}

int gbx_params_create(const char* physics_file,
                      const char* geometry,
                      const gbx_params_options* options,
                      gbx_params** out)
{
    return guarded([&] {
        if (!physics_file || !geometry || !out)
            throw std::runtime_error("null argument");
        gbx::CoreParams::Input inp;
        inp.physics_file = physics_file;
        inp.geometry = geometry_by_name(geometry);
        if (options)
        {
            inp.options.msc = options->msc != 0;
            inp.options.track_order = options->track_order;
            inp.options.rng_per_track = options->rng_per_track != 0;
            inp.options.event_tallies = options->event_tallies != 0;
            inp.options.reentrant_looping = options->reentrant_looping != 0;
            if (options->rz_field_file)
                inp.options.rz_field_file = options->rz_field_file;
            inp.options.brem_combined = options->brem_combined != 0;
            if (auto const* f = options->field_options)
            {
                gbx::FieldOptions& o = inp.options.field_options;
                o.minimum_step = f->minimum_step;
                o.delta_chord = f->delta_chord;
                o.delta_intersection = f->delta_intersection;
                o.epsilon_step = f->epsilon_step;
                o.epsilon_rel_max = f->epsilon_rel_max;
                o.errcon = f->errcon;
                o.pgrow = f->pgrow;
                o.pshrink = f->pshrink;
                o.safety = f->safety;
                o.max_stepping_increase = f->max_stepping_increase;
                o.max_stepping_decrease = f->max_stepping_decrease;
                if (f->max_nsteps <= 0 || f->max_nsteps > 32767 || f->max_substeps <= 0
                    || f->max_substeps > 32767)
                    throw std::runtime_error("invalid field driver options");
                o.max_nsteps = static_cast<short>(f->max_nsteps);
                o.max_substeps = static_cast<short>(f->max_substeps);
            }
            if (options->secondary_stack_factor != 0)
            {
                if (!(options->secondary_stack_factor > 0))
                    throw std::runtime_error("secondary_stack_factor must be positive");
                inp.options.secondary_stack_factor = options->secondary_stack_factor;
            }
            for (int i = 0; i < 3; ++i)
                inp.options.field_tesla[i] = options->field_tesla[i];
        }
        auto p = std::make_unique<gbx_params_s>();
        p->params = std::make_shared<gbx::CoreParams>(inp);
        if (options)
            p->initializer_capacity = options->initializer_capacity;
        *out = p.release();
    });
}

void gbx_params_destroy(gbx_params* params)
{
    delete params;
}

int gbx_params_num_actions(const gbx_params* params, unsigned int* num)
{
    return guarded([&] { *num = params->params->action_reg().num_actions(); });
}

int gbx_params_action_label(const gbx_params* params,
                            unsigned int action_id,
                            char* buf,
                            size_t buf_size)
{
    return guarded([&] {
        if (copy_label(params->params->action_reg().id_to_label(action_id),
                       buf,
                       buf_size))
            throw std::runtime_error("invalid label buffer");
    });
}

int gbx_params_num_detectors(const gbx_params* params, unsigned int* num)
{
    return guarded([&] { *num = params->params->host().scalars.num_detectors; });
}

int gbx_params_detector_label(const gbx_params* params,
                              unsigned int detector,
                              char* buf,
                              size_t buf_size)
{
    return guarded([&] {
        if (copy_label(params->params->host().detector_labels.at(detector),
                       buf,
                       buf_size))
            throw std::runtime_error("invalid label buffer");
    });
}

int gbx_stepper_create(gbx_params* params,
                       unsigned int num_track_slots,
                       unsigned int seed,
                       int use_graph,
                       gbx_stepper** out)
{
    return guarded([&] {
        if (!params || !out)
            throw std::runtime_error("null argument");
        gbx::StepperInput inp;
        inp.params = params->params;
        inp.num_track_slots = num_track_slots;
        inp.seed = seed;
        inp.use_graph = use_graph != 0;
        inp.initializer_capacity = params->initializer_capacity;
        auto s = std::make_unique<gbx_stepper_s>();
        s->stepper = std::make_unique<gbx::Stepper>(inp);
        if (cudaError_t err = cudaGetDevice(&s->device); err != cudaSuccess)
            throw std::runtime_error(cudaGetErrorString(err));
        if (num_track_slots <= GBX_STATIC_SCRATCH_MAX_SLOTS)
        {
            // Set up the static scratch of
            // gbx_stepper_extend_from_secondaries_static now, so that its
            // later calls do no lookup (that entry point still looks up
            // lazily if this is skipped)
            gbx::static_scratch_for_current_device();
        }
        *out = s.release();
    });
}

void gbx_stepper_destroy(gbx_stepper* stepper)
{
    delete stepper;
}

int gbx_stepper_step(gbx_stepper* stepper,
                     const gbx_primary* primaries,
                     size_t num_primaries,
                     gbx_step_result* result)
{
    return guarded([&] {
        auto& st = *stepper->stepper;
        gbx::StepperResult r;
        if (num_primaries > 0)
        {
            r = st(to_initializers(
                st.params().host().scalars, primaries, num_primaries));
        }
        else
        {
            r = st();
        }
        if (result)
            *result = to_c(r);
    });
}

int gbx_stepper_run(gbx_stepper* stepper,
                    unsigned int max_steps,
                    unsigned int batch,
                    gbx_step_result* results,
                    size_t capacity,
                    unsigned int* num_steps)
{
    return guarded([&] {
        auto recs = stepper->stepper->run_until_empty(max_steps, batch);
        for (size_t i = 0; i < recs.size() && i < capacity; ++i)
            results[i] = to_c(recs[i]);
        if (num_steps)
            *num_steps = static_cast<unsigned int>(recs.size());
    });
}

int gbx_stepper_launch_action(gbx_stepper* stepper, unsigned int action_id)
{
    return guarded([&] {
        auto& st = *stepper->stepper;
        auto const& reg = st.params().action_reg();
        if (action_id >= reg.num_actions())
            throw std::runtime_error("invalid action ID");
        auto const* sa = dynamic_cast<gbx::CoreStepActionInterface const*>(
            reg.action(action_id).get());
        if (!sa)
            throw std::runtime_error("action has no step");
        sa->step(st.params(), st.state());
        if (cudaError_t err = cudaGetLastError(); err != cudaSuccess)
            throw std::runtime_error(cudaGetErrorString(err));
    });
}

int gbx_stepper_insert_primaries(gbx_stepper* stepper,
                                 const gbx_primary* primaries,
                                 size_t num_primaries)
{
    return guarded([&] {
        auto& st = *stepper->stepper;
        auto inits = to_initializers(
            st.params().host().scalars, primaries, num_primaries);
        st.state().insert_primaries(inits.data(),
                                    static_cast<gbx::size_type>(inits.size()));
    });
}

int gbx_stepper_sorted_action_sizes(gbx_stepper* stepper,
                                    int key,
                                    unsigned int* sizes,
                                    size_t num_actions)
{
    return guarded([&] {
        if (!sizes || (key != 0 && key != 1))
            throw std::runtime_error("invalid argument");
        auto v = stepper->stepper->state().sorted_action_sizes(key);
        if (num_actions != v.size())
            throw std::runtime_error("expected one size per action");
        std::copy(v.begin(), v.end(), sizes);
    });
}

int gbx_stepper_event_live(gbx_stepper* stepper,
                           unsigned int* counts,
                           size_t num_events)
{
    return guarded([&] {
        if (num_events && !counts)
            throw std::runtime_error("null argument");
        auto v = stepper->stepper->state().event_live(
            static_cast<gbx::size_type>(num_events));
        std::copy(v.begin(), v.end(), counts);
    });
}

int gbx_stepper_event_energy_deposition(gbx_stepper* stepper,
                                        double* out,
                                        size_t num_events,
                                        int clear)
{
    return guarded([&] {
        if (num_events && !out)
            throw std::runtime_error("null argument");
        if (!stepper->stepper->params().host().scalars.event_tallies)
            throw std::runtime_error("per-event tallies are not enabled");
        auto v = stepper->stepper->state().event_energy_deposition(
            static_cast<gbx::size_type>(num_events), clear != 0);
        std::copy(v.begin(), v.end(), out);
    });
}

int gbx_stepper_event_detector_energy_deposition(gbx_stepper* stepper,
                                                 double* out,
                                                 unsigned int first_event,
                                                 size_t num_events,
                                                 int clear)
{
    return guarded([&] {
        if (!stepper || (num_events && !out))
            throw std::runtime_error("null argument");
        if (!stepper->stepper->params().host().scalars.event_tallies)
            throw std::runtime_error("per-event tallies are not enabled");
        auto v = stepper->stepper->state().event_detector_energy_deposition(
            first_event, static_cast<gbx::size_type>(num_events), clear != 0);
        std::copy(v.begin(), v.end(), out);
    });
}

int gbx_stepper_generate_primaries(gbx_stepper* stepper,
                                   const gbx_primary_generator_options* options,
                                   unsigned int first_event)
{
    return guarded([&] {
        if (!stepper || !options)
            throw std::runtime_error("null argument");
        gbx_primary_generator_options const& o = *options;
        if (o.num_pdg == 0 || o.num_pdg > 8)
            throw std::runtime_error("primary generator needs 1 to 8 PDG codes");
        if (o.num_events == 0 || o.primaries_per_event == 0)
            throw std::runtime_error("primary generator needs events and primaries");
        // The reference's samplers (make_*_sampler,
        // src/celeritas/phys/PrimaryGeneratorOptions.cc)
        auto invalid = [](char const* dist, char const* sampler) {
            return std::runtime_error(std::string("invalid distribution type '") + dist
                                      + "' for " + sampler);
        };
        auto name = [](int d) {
            return d == GBX_DIST_DELTA       ? "delta"
                   : d == GBX_DIST_ISOTROPIC ? "isotropic"
                   : d == GBX_DIST_BOX       ? "box"
                                             : "unknown";
        };
        if (o.energy_distribution != GBX_DIST_DELTA)
            throw invalid(name(o.energy_distribution), "energy");
        if (o.position_distribution != GBX_DIST_DELTA
            && o.position_distribution != GBX_DIST_BOX)
            throw invalid(name(o.position_distribution), "position");
        if (o.direction_distribution != GBX_DIST_DELTA
            && o.direction_distribution != GBX_DIST_ISOTROPIC)
            throw invalid(name(o.direction_distribution), "direction");
        if (!(o.energy[0] > 0))
            throw std::runtime_error("primary energy must be positive");

        gbx::PrimaryGeneratorData g{};
        g.seed = o.seed;
        g.num_particles = o.num_pdg;
        auto const& particles = stepper->stepper->params().host().particles;
        for (unsigned int i = 0; i < o.num_pdg; ++i)
        {
            g.particle_ids[i] = gbx::invalid_id;
            for (gbx::size_type p = 0; p < particles.size(); ++p)
            {
                if (particles[p].pdg == o.pdg[i])
                    g.particle_ids[i] = p;
            }
            if (g.particle_ids[i] == gbx::invalid_id)
                throw std::runtime_error("no particle with PDG code "
                                         + std::to_string(o.pdg[i]));
        }
        g.primaries_per_event = o.primaries_per_event;
        g.first_event = first_event;
        g.num_events = o.num_events;
        g.energy_dist = o.energy_distribution;
        g.energy = o.energy[0];
        g.position_dist = o.position_distribution;
        for (int i = 0; i < 6; ++i)
            g.position[i] = o.position[i];
        g.direction_dist = o.direction_distribution;
        for (int i = 0; i < 3; ++i)
            g.direction[i] = o.direction[i];
        stepper->stepper->state().generate_primaries(g);
    });
}

static_assert(GBX_DIST_BOX == gbx::dist_box && GBX_DIST_ISOTROPIC == gbx::dist_isotropic,
              "distribution values differ");

int gbx_stepper_set_step_output(gbx_stepper* stepper,
                                unsigned int selection,
                                int nonzero_energy_deposition,
                                size_t capacity)
{
    return guarded([&] {
        if (!stepper)
            throw std::runtime_error("null argument");
        if (capacity > size_t(std::numeric_limits<gbx::size_type>::max()))
            throw std::runtime_error("step output capacity too large");
        stepper->stepper->set_step_output(
            selection, nonzero_energy_deposition != 0, static_cast<gbx::size_type>(capacity));
    });
}

int gbx_stepper_read_step_output(gbx_stepper* stepper,
                                 const gbx_step_hits* out,
                                 size_t* num_hits)
{
    return guarded([&] {
        if (!stepper || !out || !num_hits)
            throw std::runtime_error("null argument");
        gbx::StepHitsRef dst;
        dst.capacity = static_cast<gbx::size_type>(
            std::min<size_t>(out->capacity, std::numeric_limits<gbx::size_type>::max()));
        dst.step = out->step;
        dst.detector = out->detector;
        dst.track_id = out->track_id;
        dst.event_id = out->event_id;
        dst.parent_id = out->parent_id;
        dst.track_step_count = out->track_step_count;
        dst.particle = out->particle;
        dst.step_length = out->step_length;
        dst.energy_deposition = out->energy_deposition;
        dst.pre_time = out->pre_time;
        dst.pre_pos = out->pre_pos;
        dst.pre_dir = out->pre_dir;
        dst.pre_energy = out->pre_energy;
        dst.post_time = out->post_time;
        dst.post_pos = out->post_pos;
        dst.post_dir = out->post_dir;
        dst.post_energy = out->post_energy;
        *num_hits = stepper->stepper->state().read_step_output(dst);
    });
}

static_assert(GBX_STEP_ALL == gbx::step_select_all, "step selection bits differ");
static_assert(GBX_STEP_ENERGY_DEPOSITION == gbx::step_energy_deposition,
              "step selection bits differ");
static_assert(sizeof(unsigned int) == sizeof(gbx::size_type), "index type differs");

int gbx_stepper_set_tuning(gbx_stepper* stepper, const char* name, long long value)
{
    return guarded([&] {
        if (!name)
            throw std::runtime_error("null argument");
        stepper->stepper->set_tuning(name, value);
    });
}

int gbx_stepper_get_tuning(gbx_stepper* stepper, const char* name, long long* value)
{
    return guarded([&] {
        if (!name || !value)
            throw std::runtime_error("null argument");
        *value = stepper->stepper->tuning(name);
    });
}

static_assert(GBX_STATIC_SCRATCH_MAX_SLOTS == gbx::static_scratch_max_slots,
              "public and internal static scratch limits differ");

int gbx_stepper_extend_from_secondaries_static(gbx_stepper* stepper)
{
    return guarded([&] {
        if (!stepper)
            throw std::runtime_error("null argument");
        int device = -1;
        if (cudaError_t err = cudaGetDevice(&device); err != cudaSuccess)
            throw std::runtime_error(cudaGetErrorString(err));
        if (device != stepper->device)
        {
            throw std::runtime_error(
                "the stepper was created on device " + std::to_string(stepper->device)
                + " but device " + std::to_string(device)
                + " is current: make the stepper's device current first");
        }
        auto& state = stepper->stepper->state();
        gbx::launch_extend_from_secondaries_static(state.context(), state.stream());
        if (cudaError_t err = cudaGetLastError(); err != cudaSuccess)
            throw std::runtime_error(cudaGetErrorString(err));
    });
}

int gbx_libm_evaluate(int function, const double* x, double* y, size_t n)
{
    return guarded([&] {
        if (function < GBX_LIBM_EXP || function > GBX_LIBM_CBRT)
            throw std::runtime_error("unknown elementary function");
        if (n == 0)
            return;
        if (!x || !y)
            throw std::runtime_error("null argument");
        double* buf = nullptr;
        auto check = [&buf](cudaError_t err) {
            if (err != cudaSuccess)
            {
                if (buf)
                    cudaFree(buf);
                throw std::runtime_error(cudaGetErrorString(err));
            }
        };
        check(gbx::device_malloc(reinterpret_cast<void**>(&buf), 2 * n * sizeof(double)));
        check(cudaMemcpy(buf, x, n * sizeof(double), cudaMemcpyHostToDevice));
        unsigned int const blocks
            = static_cast<unsigned int>(std::min<size_t>((n + 255) / 256, 4096));
        libm_evaluate_kernel<<<blocks, 256>>>(function, buf, buf + n, n);
        check(cudaGetLastError());
        check(cudaMemcpy(y, buf + n, n * sizeof(double), cudaMemcpyDeviceToHost));
        check(cudaFree(buf));
    });
}

int gbx_device_allocations(unsigned long long* count)
{
    return guarded([&] {
        if (!count)
            throw std::runtime_error("null argument");
        *count = gbx::device_allocation_count();
    });
}

int gbx_stepper_warm_up(gbx_stepper* stepper)
{
    return guarded([&] {
        if (!stepper)
            throw std::runtime_error("null argument");
        stepper->stepper->warm_up();
    });
}

int gbx_stepper_kill_active(gbx_stepper* stepper)
{
    return guarded([&] { stepper->stepper->kill_active(); });
}

int gbx_stepper_reseed(gbx_stepper* stepper, unsigned long long event_id)
{
    return guarded([&] { stepper->stepper->reseed(event_id); });
}

int gbx_stepper_synchronize(gbx_stepper* stepper)
{
    return guarded([&] {
        if (cudaError_t err = cudaStreamSynchronize(stepper->stepper->state().stream());
            err != cudaSuccess)
            throw std::runtime_error(cudaGetErrorString(err));
    });
}

int gbx_stepper_stream(gbx_stepper* stepper, void** stream)
{
    return guarded([&] { *stream = stepper->stepper->state().stream(); });
}

int gbx_stepper_step_kernels(gbx_stepper* stepper, unsigned int* num_kernels)
{
    return guarded([&] { *num_kernels = stepper->stepper->graph_kernel_count(); });
}

int gbx_stepper_set_action_times(gbx_stepper* stepper, int enable)
{
    return guarded([&] { stepper->stepper->set_action_times(enable != 0); });
}

int gbx_stepper_action_times(gbx_stepper* stepper,
                             double* milliseconds,
                             unsigned int* launches,
                             size_t capacity)
{
    return guarded([&] {
        auto& seq = stepper->stepper->action_sequence();
        auto ms = seq.action_times();
        auto nl = seq.action_launches();
        for (size_t i = 0; i < ms.size() && i < capacity; ++i)
        {
            if (milliseconds)
                milliseconds[i] = ms[i];
            if (launches)
                launches[i] = nl[i];
        }
        seq.reset_action_times();
    });
}

int gbx_stepper_energy_deposition(gbx_stepper* stepper,
                                  double* out,
                                  size_t num_detectors)
{
    return guarded([&] {
        auto e = stepper->stepper->energy_deposition();
        if (num_detectors < e.size())
            throw std::runtime_error("output buffer too small");
        std::memcpy(out, e.data(), e.size() * sizeof(double));
    });
}

int gbx_stepper_clear_energy_deposition(gbx_stepper* stepper)
{
    return guarded([&] { stepper->stepper->clear_energy_deposition(); });
}

int gbx_stepper_copy_state(gbx_stepper* stepper,
                           const char* field,
                           void* host,
                           size_t nbytes,
                           int direction)
{
    return guarded([&] {
        auto& st = stepper->stepper->state();
        FieldRef f = find_field(st, field);
        if (nbytes > f.elem * f.count)
            throw std::runtime_error("copy exceeds state array size");
        cudaError_t err;
        if (direction > 0)
            err = cudaMemcpyAsync(f.ptr, host, nbytes, cudaMemcpyHostToDevice, st.stream());
        else
            err = cudaMemcpyAsync(host, f.ptr, nbytes, cudaMemcpyDeviceToHost, st.stream());
        if (err == cudaSuccess)
            err = cudaStreamSynchronize(st.stream());
        if (err != cudaSuccess)
            throw std::runtime_error(cudaGetErrorString(err));
    });
}

int gbx_stepper_state_info(gbx_stepper* stepper,
                           const char* field,
                           size_t* elem_bytes,
                           size_t* count)
{
    return guarded([&] {
        FieldRef f = find_field(stepper->stepper->state(), field);
        *elem_bytes = f.elem;
        *count = f.count;
    });
}

}  // extern "C"
