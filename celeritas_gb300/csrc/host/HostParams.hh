// Host-side construction of the stepping-loop parameters from the physics
// input file and a geometry description.
#pragma once

#include <string>
#include <vector>

#include "../gbx/Data.hh"

namespace gbx
{
//! An axis-aligned box volume of the geometry description
struct BoxSpec
{
    std::string label;
    double lo[3];
    double hi[3];
    size_type material;
};

//! Boxes (non-overlapping, sorted along the stacking axis) in a world box
struct GeometrySpec
{
    std::string name;
    double world_lo[3];
    double world_hi[3];
    size_type background_material{0};
    std::vector<BoxSpec> boxes;
    int stack_axis{2};
};

//! Sampling calorimeter: layers of (absorber, gap) along +z
GeometrySpec make_calorimeter_geometry(int num_layers = 50,
                                       double absorber = 0.23,
                                       double gap = 0.57,
                                       double half_xy = 20.0);

//! Options mirroring celer-sim's RunnerInput physics/transport knobs
struct ParamsOptions
{
    double secondary_stack_factor{3};
    bool brem_combined{false};
    //! Urban multiple scattering for e-/e+
    bool msc{false};
    //! Uniform magnetic field [tesla]; zero for straight-line transport
    double field_tesla[3]{0, 0, 0};
    //! TrackOrder policy (none or one of the action sorts)
    unsigned int track_order{0};
};

//! All parameter tables in host memory
struct HostParams
{
    std::vector<real_type> reals;  //!< Physics tables (FP32 in the mixed build)
    std::vector<size_type> ints;
    std::vector<ParticleRecord> particles;
    std::vector<ElementRecord> elements;
    std::vector<MaterialRecord> materials;
    std::vector<UrbanFluctRecord> fluct;
    std::vector<real_type> cutoffs;
    std::vector<ProcessGroup> groups;
    std::vector<XsGrid> grids;
    std::vector<LivermoreElement> lv_elements;
    std::vector<LivermoreShell> lv_shells;
    std::vector<SBElementTable> sb_tables;
    std::vector<RelBremElementRecord> rb_elements;
    std::vector<UrbanMscMaterialRecord> msc_materials;
    std::vector<UrbanMscParMatRecord> msc_par_mat;
    std::vector<LoopingRecord> looping;
    // Geometry
    std::vector<PlaneRecord> planes;
    std::vector<BoxVolume> boxes;
    std::vector<size_type> neighbor_offset;
    std::vector<size_type> neighbors;
    std::vector<size_type> volume_material;
    std::vector<size_type> volume_detector;
    std::vector<std::string> volume_labels;
    std::vector<std::string> detector_labels;
    std::vector<std::string> action_labels;
    std::vector<std::string> material_labels;

    //! Scalars and IDs; pointer members are filled by make_host_view
    ParamsData scalars{};
};

//! Build parameters (throws std::runtime_error on invalid input)
HostParams build_params(std::string const& physics_path,
                        GeometrySpec const& geo,
                        ParamsOptions const& opts);

//! View with pointers into the host vectors
ParamsData make_host_view(HostParams const& hp);

}  // namespace gbx
