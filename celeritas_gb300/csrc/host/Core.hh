// Host-side stepping-loop API with the reference's names and semantics:
// StepActionOrder, ActionInterface / CoreStepActionInterface, ActionRegistry,
// ActionSequence, CoreParams / CoreState and Stepper
// (src/corecel/sys/ActionInterface.hh:29-186, ActionRegistry.hh:42-105,
//  src/celeritas/global/ActionSequence.cc:37-138, CoreParams.hh:68-172,
//  CoreState.hh:74-182, Stepper.hh:43-201).
//
// Each action's device step() launches one hand-written sm_103a kernel
// through the C-ABI launch layer; state, counters and tables stay on the
// device, and steps without primaries are replayed from a CUDA graph.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

#include "../device/Kernels.cuh"
#include "HostParams.hh"

namespace gbx
{
class CoreParams;
class CoreState;

//---------------------------------------------------------------------------//
//! Ordering of step actions within a step (ActionInterface.hh:29-45)
enum class StepActionOrder
{
    generate,
    start,
    user_start,
    sort_start,
    pre,
    user_pre,
    sort_pre,
    along,
    sort_along,
    pre_post,
    sort_pre_post,
    post,
    user_post,
    end,
    size_
};

using ActionId = size_type;

//! Base class for all actions (ActionInterface.hh:78-96)
class ActionInterface
{
  public:
    virtual ~ActionInterface() = default;
    virtual ActionId action_id() const = 0;
    virtual std::string_view label() const = 0;
    virtual std::string_view description() const = 0;
};

//! An action that acts on the core state every step (CoreStepActionInterface)
class CoreStepActionInterface : public virtual ActionInterface
{
  public:
    virtual StepActionOrder order() const = 0;
    //! Launch the action's kernel(s) on the state's stream
    virtual void step(CoreParams const& params, CoreState& state) const = 0;
};

//! Action with fixed ID, label and description (ConcreteAction)
class ConcreteAction : public virtual ActionInterface
{
  public:
    ConcreteAction(ActionId id, std::string label, std::string description)
        : id_(id), label_(std::move(label)), description_(std::move(description))
    {
    }
    ActionId action_id() const final { return id_; }
    std::string_view label() const final { return label_; }
    std::string_view description() const final { return description_; }

  private:
    ActionId id_;
    std::string label_;
    std::string description_;
};

//! Action with no step (implicit post-step limits such as "eloss-range")
class ImplicitAction final : public ConcreteAction
{
  public:
    using ConcreteAction::ConcreteAction;
};

//! Sequential registry of actions (ActionRegistry.hh:42-105)
class ActionRegistry
{
  public:
    using SPConstAction = std::shared_ptr<ActionInterface const>;

    ActionId next_id() const { return static_cast<ActionId>(actions_.size()); }
    void insert(SPConstAction action);
    SPConstAction const& action(ActionId id) const { return actions_.at(id); }
    std::string const& id_to_label(ActionId id) const { return labels_.at(id); }
    ActionId find_action(std::string_view label) const;
    ActionId num_actions() const { return static_cast<ActionId>(actions_.size()); }
    bool empty() const { return actions_.empty(); }

  private:
    std::vector<SPConstAction> actions_;
    std::vector<std::string> labels_;
};

//---------------------------------------------------------------------------//
//! Immutable problem data on host and device (CoreParams)
class CoreParams
{
  public:
    struct Input
    {
        std::string physics_file;
        GeometrySpec geometry;
        ParamsOptions options;
    };

    explicit CoreParams(Input const& inp);
    ~CoreParams();
    CoreParams(CoreParams const&) = delete;
    CoreParams& operator=(CoreParams const&) = delete;

    HostParams const& host() const { return host_; }
    ParamsData const& device_ref() const { return device_; }
    ActionRegistry const& action_reg() const { return *actions_; }
    ActionRegistry& action_reg() { return *actions_; }

  private:
    HostParams host_;
    ParamsData device_{};
    void* device_storage_{nullptr};
    std::shared_ptr<ActionRegistry> actions_;
};

//---------------------------------------------------------------------------//
//! Per-stream mutable track state on the device (CoreState)
class CoreState
{
  public:
    CoreState(CoreParams const& params,
              size_type num_track_slots,
              unsigned int seed,
              size_type initializer_capacity,
              size_type max_events,
              cudaStream_t stream);
    ~CoreState();
    CoreState(CoreState const&) = delete;
    CoreState& operator=(CoreState const&) = delete;

    size_type size() const { return ref_.size; }
    StateData const& ref() const { return ref_; }
    LaunchContext const& context() const { return ctx_; }
    cudaStream_t stream() const { return stream_; }

    //! Stage primaries on the device for the next generate action
    void insert_primaries(TrackInitializer const* host_primaries, size_type n);
    //! Sample primaries on the device into the staging buffer for the next
    //! generate action (PrimaryGenerator; no host copy). The events must
    //! have no primaries yet. 'gen' holds particle indices of these params.
    void generate_primaries(PrimaryGeneratorData gen);
    size_type pending_primaries() const { return pending_primaries_; }
    void clear_pending_primaries() { pending_primaries_ = 0; }

    //! Copy the device counters to the host (synchronizes the stream)
    Counters counters() const;
    //! Number of completed steps recorded on the device
    size_type step_index() const;
    //! Launch tuning: "along_block_size" (64, 128, 256, 512),
    //! "along_persistent" (0/1), "sort" (0/1: whether the action sorts run),
    //! "partition_slots" (0/1: charged tracks fill vacancies from the front
    //! of the list, neutral ones from the back; per-track streams only),
    //! "sort_material" (bit 0: the along-step sort orders the charged
    //! tracks by material too, bit 1: the neutral ones)
    void set_tuning(std::string const& name, long long value);
    long long tuning(std::string const& name) const;

    //! Reseed every slot's random state for an event and restart the
    //! per-event track IDs (Stepper::reseed)
    void reseed(unsigned long long event_id);

    //! Live tracks (slots and queued initializers) per event [0, n)
    std::vector<size_type> event_live(size_type n) const;
    //! Tracks in each action's range of the last action sort by 'key' (0:
    //! along-step action, 1: step-limit action), indexed by action ID
    std::vector<size_type> sorted_action_sizes(int key) const;
    //! Energy deposited in detectors per event [0, n); optionally cleared
    std::vector<double> event_energy_deposition(size_type n, bool clear);
    //! Energy deposited in each detector per event, events [first, first +
    //! n), event-major ([n][detectors]); optionally cleared
    std::vector<double>
    event_detector_energy_deposition(size_type first, size_type n, bool clear);
    //! Read the step log entries [first, first + n)
    std::vector<StepRecord> step_log(size_type first, size_type n) const;
    size_type log_capacity() const { return ctx_.log_capacity; }

    //! Collect the hits of every step (StepCollector with DetectorSteps):
    //! the selected data of each track step in a detector volume, dropping
    //! steps without deposition if asked, into device buffers of 'capacity'
    //! records that the host empties with read_step_output. Zero capacity
    //! turns the output off. Allocates the buffers (outside the step loop).
    void set_step_output(unsigned int selection,
                         bool nonzero_energy_deposition,
                         size_type capacity);
    StepHitsRef const& step_output() const { return ctx_.hits; }
    //! Copy the records held on the device into the arrays of 'out' (host
    //! memory, null where not wanted; 'out.capacity' entries each), empty the
    //! device buffers and return the number of records. Throws if the device
    //! buffers overflowed since the last read (they are emptied) or if 'out'
    //! is too small (they are kept).
    size_type read_step_output(StepHitsRef const& out);

  private:
    StateData ref_{};
    LaunchContext ctx_{};
    int sort_material_ = 0;  //!< Tuning value of "sort_material"
    void* storage_{nullptr};
    void* hits_storage_{nullptr};
    TrackInitializer* pinned_primaries_{nullptr};
    size_type pinned_capacity_{0};
    size_type pending_primaries_{0};
    unsigned int seed_{0};
    size_type ndet_{0};
    //! Primaries inserted so far per event (seeds of per-track streams)
    std::unordered_map<size_type, size_type> primaries_per_event_;
    cudaStream_t stream_{nullptr};
};

//---------------------------------------------------------------------------//
//! Ordered list of step actions (ActionSequence)
class ActionSequence
{
  public:
    explicit ActionSequence(ActionRegistry const& reg);
    ~ActionSequence();
    void step(CoreParams const& params, CoreState& state) const;
    std::vector<CoreStepActionInterface const*> const& actions() const
    {
        return actions_;
    }

    //! Record device time per action with CUDA events on the state's stream
    //! (the reference's StepperInput::action_times; disables graph replay)
    void enable_action_times(bool enable);
    bool action_times_enabled() const { return timing_; }
    //! Accumulated device milliseconds per action ID (synchronizes)
    std::vector<double> action_times() const;
    //! Number of timed launches per action ID
    std::vector<size_type> action_launches() const { return launches_; }
    void reset_action_times();

  private:
    std::vector<CoreStepActionInterface const*> actions_;
    size_type num_ids_{0};
    bool timing_{false};
    mutable std::vector<cudaEvent_t> start_;
    mutable std::vector<cudaEvent_t> stop_;
    mutable std::vector<double> elapsed_;
    mutable std::vector<size_type> launches_;
    mutable std::vector<bool> pending_;
    void collect() const;
};

//! Stepper input (Stepper.hh:43-55)
struct StepperInput
{
    std::shared_ptr<CoreParams const> params;
    size_type stream_id{0};
    size_type num_track_slots{0};
    unsigned int seed{0};
    size_type initializer_capacity{0};  //!< default 4 x slots (min 2^20)
    size_type max_events{1u << 16};
    bool use_graph{true};
};

//! Step counts (Stepper.hh:61-70)
struct StepperResult
{
    size_type generated{0};
    size_type queued{0};
    size_type active{0};
    size_type alive{0};
    explicit operator bool() const { return queued > 0 || alive > 0; }
};

//! Step the track state, the reference's Stepper<MemSpace::device>
class Stepper
{
  public:
    explicit Stepper(StepperInput const& input);
    ~Stepper();

    //! Take one step with primaries
    StepperResult operator()(std::vector<TrackInitializer> const& primaries);
    //! Take one step
    StepperResult operator()();
    //! Take up to 'max_steps' steps until the state is empty; record counts
    std::vector<StepperResult> run_until_empty(size_type max_steps,
                                               size_type batch = 16);
    //! Kill all tracks in flight
    void kill_active();
    //! Reseed the random states of all slots for an event and restart its
    //! track IDs (Stepper::reseed, src/celeritas/global/Stepper.cc:194-201)
    void reseed(unsigned long long event_id);
    //! One step over the empty state, loading every kernel and capturing
    //! the step graph of each sort state (Stepper::warm_up,
    //! src/celeritas/global/Stepper.cc:105-115)
    void warm_up();

    CoreState& state() { return *state_; }
    CoreParams const& params() const { return *params_; }
    ActionSequence const& actions() const { return *actions_; }

    //! Kernel nodes in the captured step graph (captures it if needed)
    size_type graph_kernel_count();

    //! Time each action's kernels with CUDA events (action_times)
    void set_action_times(bool enable) { actions_->enable_action_times(enable); }
    ActionSequence& action_sequence() { return *actions_; }

    //! Energy deposition per detector [MeV] (synchronizes)
    std::vector<double> energy_deposition() const;
    void clear_energy_deposition();

    //! Step output (see CoreState::set_step_output); drops the captured
    //! step graphs, whose gather action gains or loses the hit kernels
    void set_step_output(unsigned int selection,
                         bool nonzero_energy_deposition,
                         size_type capacity);

    //! Launch tuning (see CoreState::set_tuning) plus "sort_threshold": the
    //! action sorts run only in steps that start with at least this many
    //! active tracks (0: always). Drops the captured step graphs.
    void set_tuning(std::string const& name, long long value);
    long long tuning(std::string const& name) const;

  private:
    std::shared_ptr<CoreParams const> params_;
    std::unique_ptr<CoreState> state_;
    std::unique_ptr<ActionSequence> actions_;
    cudaStream_t stream_{nullptr};
    // Captured step graphs, without (0) and with (1) the action sorts
    cudaGraphExec_t graph_exec_[2]{nullptr, nullptr};
    cudaGraph_t graph_[2]{nullptr, nullptr};
    bool use_graph_{true};
    long long sort_threshold_{0};
    size_type last_active_{0};

    void clear_graphs();
    void update_sort_policy();

    void launch_steps(size_type count);
    void build_graph();
    StepperResult read_record(size_type index) const;
};

//! cudaMalloc, counted: every device allocation of the library goes
//! through here
cudaError_t device_malloc(void** ptr, std::size_t bytes);
//! Number of device allocations made so far by this library (all devices)
unsigned long long device_allocation_count();

//! Register the stepping-loop actions in the reference's order and return
//! the list (CoreParams::build_actions, PhysicsParams actions, models)
void register_core_actions(ActionRegistry* reg,
                           bool uniform_field,
                           bool rz_map,
                           unsigned int track_order,
                           bool brem_combined = false);

}  // namespace gbx
