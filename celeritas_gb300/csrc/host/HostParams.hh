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

//! Cylindrical shell about the z axis: r_in < r < r_out, z_lo < z < z_hi
struct ShellSpec
{
    std::string label;
    double r_in;
    double r_out;
    double z_lo;
    double z_hi;
    size_type material;
};

//! Non-overlapping volumes in a world box: either boxes (sorted along z) or
//! cylindrical shells
struct GeometrySpec
{
    std::string name;
    double world_lo[3];
    double world_hi[3];
    size_type background_material{0};
    std::vector<BoxSpec> boxes;
    std::vector<ShellSpec> shells;
};

//! Sampling calorimeter: layers of (absorber, gap) along +z
GeometrySpec make_calorimeter_geometry(int num_layers = 50,
                                       double absorber = 0.23,
                                       double gap = 0.57,
                                       double half_xy = 20.0);

//! CMS-like detector of concentric shells about z: 10 silicon layers
//! (0.3 mm, r = 4-110 cm, |z| < 270 cm), a PbWO4 barrel (r = 129-152 cm,
//! |z| < 300 cm) and 17 brass (5 cm) / plastic scintillator (0.4 cm) pairs
//! (r = 180-295 cm, |z| < 300 cm) in a vacuum world box. Materials: 0
//! vacuum, 1 Si, 2 PbWO4, 3 brass, 4 scintillator.
GeometrySpec make_cms_geometry();

//! Geometry from a text file: a 'gbx-geometry 1' line, then one record per
//! line ('#' starts a comment), lengths in cm, materials as indices of the
//! physics file's materials:
//!   world <lo_x> <lo_y> <lo_z> <hi_x> <hi_y> <hi_z>
//!   background <material>                      (default 0)
//!   box <label> <material> <lo_x> <lo_y> <lo_z> <hi_x> <hi_y> <hi_z>
//!   shell <label> <material> <r_in> <r_out> <z_lo> <z_hi>
//! Boxes are axis-aligned; shells are cylindrical about z. A file holds
//! boxes or shells, non-overlapping and inside the world box, as ORANGE's
//! unit built from BoxShape and CylinderSolid objects would.
GeometrySpec read_geometry_file(std::string const& path);

//! Geometry by name ("calo", "cms") or from a geometry file
GeometrySpec make_geometry(std::string const& name);

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
    //! Per-track random streams (results independent of the other events)
    bool rng_per_track{false};
    //! Per-event energy-deposition tallies
    bool event_tallies{false};
    //! A reentrant boundary step keeps the looping-step count
    bool reentrant_looping{false};
    //! R-Z field map file (empty: none); excludes a uniform field
    std::string rz_field_file;
    //! Field-driver options (RunnerInput::field_options)
    FieldOptions field_options;
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
    std::vector<std::uint32_t> rng_jump;  //!< [2][32][5] jump polynomials
    std::vector<FieldMapElement> rzmap;  //!< R-Z field map nodes
    std::vector<FieldMapElementF> rzmap_f;  //!< The nodes rounded to FP32
    RZMapData rzmap_desc{};  //!< Grids, and the nodes in host memory
    // Geometry
    std::vector<SurfaceRecord> surfaces;
    std::vector<VolumeRecord> volumes;
    std::vector<size_type> neighbor_offset;
    std::vector<size_type> neighbors;
    std::vector<size_type> sorted_surfaces;  //!< By kind, then value
    std::vector<float> sorted_key;
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
