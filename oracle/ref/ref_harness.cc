// Golden-vector harness for the CPU oracle: drives the reference's own host
// stepping loop (Stepper<MemSpace::host>, src/celeritas/global/Stepper.cc:125-168)
// on the synthetic physics file and the geometries that the GB300 path uses,
// and prints per-step counters and per-volume energy deposition.
//
// Problem set-up follows celer-sim's Runner::build_core_params
// (app/celer-sim/Runner.cc:281-446); the loop follows Transporter::operator()
// (app/celer-sim/Transporter.cc:84-179).
//
// This file is test infrastructure: it links the reference library built by
// the Makefile beside it and is never part of the shipped GB300 path.
//
// Usage:
//   ref_harness run <physics.txt> <geometry> <primaries.txt> <num_slots>
//               <seed> [--field Bx By Bz] [--msc] [--steps N] [--track-order N] [--trace]
//               [--brem-combined] [--rz-field FILE] [--hits] [--reseed N]
//               [--field-option NAME VALUE]...
//   ref_harness bench <physics.txt> <geometry> <primaries.txt> <num_slots>
//               <seed> [--threads T] [--field Bx By Bz] [--msc] [--max-steps N]
//   ref_harness geo <physics.txt> <geometry>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "corecel/data/CollectionStateStore.hh"
#include "corecel/io/Label.hh"
#include "corecel/io/OutputRegistry.hh"
#include "corecel/sys/ActionRegistry.hh"
#include "geocel/GeoParamsOutput.hh"
#include "orange/OrangeData.hh"
#include "orange/OrangeInput.hh"
#include "orange/OrangeParams.hh"
#include "orange/OrangeTypes.hh"
#include "orange/orangeinp/CsgObject.hh"
#include "orange/orangeinp/InputBuilder.hh"
#include "orange/orangeinp/IntersectRegion.hh"
#include "orange/orangeinp/Shape.hh"
#include "orange/orangeinp/Transformed.hh"
#include "orange/orangeinp/Solid.hh"
#include "orange/orangeinp/UnitProto.hh"
#include "orange/transform/VariantTransform.hh"
#include "celeritas/Quantities.hh"
#include "celeritas/Units.hh"
#include "celeritas/em/params/UrbanMscParams.hh"
#include "celeritas/field/FieldDriverOptions.hh"
#include "celeritas/field/UniformFieldData.hh"
#include "celeritas/geo/GeoMaterialParams.hh"
#include "celeritas/geo/GeoParams.hh"
#include "celeritas/global/ActionSequence.hh"
#include "celeritas/global/CoreParams.hh"
#include "celeritas/global/CoreState.hh"
#include "celeritas/global/CoreTrackView.hh"
#include "celeritas/global/Stepper.hh"
#include "celeritas/global/alongstep/AlongStepGeneralLinearAction.hh"
#include "celeritas/global/alongstep/AlongStepUniformMscAction.hh"
#include "celeritas/global/alongstep/AlongStepRZMapFieldMscAction.hh"
#include "celeritas/field/RZMapFieldInput.hh"
#include "celeritas/io/ImportData.hh"
#include "celeritas/mat/MaterialParams.hh"
#include "celeritas/phys/CutoffParams.hh"
#include "celeritas/phys/ParticleParams.hh"
#include "celeritas/phys/PhysicsParams.hh"
#include "celeritas/phys/Primary.hh"
#include "celeritas/phys/ProcessBuilder.hh"
#include "celeritas/random/RngParams.hh"
#include "celeritas/track/ExtendFromPrimariesAction.hh"
#include "celeritas/track/SimParams.hh"
#include "celeritas/track/TrackInitParams.hh"
#include "celeritas/user/DetectorSteps.hh"
#include "celeritas/user/SimpleCalo.hh"
#include "celeritas/user/StepCollector.hh"
#include "celeritas/user/StepInterface.hh"

using namespace celeritas;

namespace
{
//---------------------------------------------------------------------------//
// Key/value physics file ("key count v0 v1 ...")
//---------------------------------------------------------------------------//
struct KvFile
{
    std::map<std::string, std::vector<std::string>> records;

    explicit KvFile(std::string const& path)
    {
        std::ifstream in(path);
        if (!in)
        {
            throw std::runtime_error("cannot open " + path);
        }
        std::string line;
        while (std::getline(in, line))
        {
            std::istringstream ss(line);
            std::string key;
            std::size_t n = 0;
            if (!(ss >> key >> n))
                continue;
            std::vector<std::string> vals(n);
            for (auto& v : vals)
                ss >> v;
            records[key] = std::move(vals);
        }
    }
    bool has(std::string const& k) const { return records.count(k) > 0; }
    std::vector<std::string> const& get(std::string const& k) const
    {
        auto it = records.find(k);
        if (it == records.end())
            throw std::runtime_error("missing key " + k);
        return it->second;
    }
    std::vector<double> dbl(std::string const& k) const
    {
        std::vector<double> r;
        for (auto const& s : get(k))
            r.push_back(std::strtod(s.c_str(), nullptr));
        return r;
    }
    double d(std::string const& k) const { return dbl(k).at(0); }
    long i(std::string const& k) const { return std::stol(get(k).at(0)); }
    std::string s(std::string const& k) const { return get(k).at(0); }
};

ImportPhysicsVector log_vector(KvFile const& kv, std::string const& key)
{
    ImportPhysicsVector v;
    v.vector_type = ImportPhysicsVectorType::log;
    v.x = kv.dbl(key + ".x");
    v.y = kv.dbl(key + ".y");
    return v;
}

//---------------------------------------------------------------------------//
// Synthetic physics file -> ImportData
//---------------------------------------------------------------------------//
ImportData load_import(KvFile const& kv, bool with_msc)
{
    ImportData data;
    data.units = "cgs";

    long nel = kv.i("elements");
    for (long i = 0; i < nel; ++i)
    {
        ImportElement el;
        auto p = "element." + std::to_string(i);
        el.name = kv.s(p + ".name");
        el.atomic_number = kv.i(p + ".z");
        el.atomic_mass = kv.d(p + ".a");
        data.elements.push_back(el);
    }
    long nmat = kv.i("materials");
    for (long i = 0; i < nmat; ++i)
    {
        auto p = "material." + std::to_string(i);
        ImportGeoMaterial gm;
        gm.name = kv.s(p + ".name");
        auto st = kv.s(p + ".state");
        gm.state = st == "solid"    ? ImportMaterialState::solid
                   : st == "liquid" ? ImportMaterialState::liquid
                                    : ImportMaterialState::gas;
        gm.temperature = kv.d(p + ".temperature");
        gm.number_density = kv.d(p + ".number_density");
        auto els = kv.dbl(p + ".elements");
        auto fr = kv.dbl(p + ".fractions");
        for (std::size_t j = 0; j < els.size(); ++j)
        {
            gm.elements.push_back(
                {static_cast<unsigned int>(els[j]), fr[j]});
        }
        data.geo_materials.push_back(gm);

        ImportPhysMaterial pm;
        pm.geo_material_id = i;
        for (int pdg : {11, -11, 22})
        {
            auto c = kv.dbl(p + ".cut." + std::to_string(pdg));
            pm.pdg_cutoffs[pdg] = ImportProductionCut{c[0], c[1]};
        }
        data.phys_materials.push_back(pm);
    }

    long npar = kv.i("particles");
    for (long i = 0; i < npar; ++i)
    {
        auto const& v = kv.get("particle." + std::to_string(i));
        ImportParticle ip;
        ip.name = v[0];
        ip.pdg = std::stoi(v[1]);
        ip.mass = std::strtod(v[2].c_str(), nullptr);
        ip.charge = std::strtod(v[3].c_str(), nullptr);
        ip.spin = std::strtod(v[4].c_str(), nullptr);
        ip.lifetime = -1;
        ip.is_stable = true;
        data.particles.push_back(ip);
    }

    auto make_table = [&](std::string const& prefix, ImportTableType tt) {
        ImportPhysicsTable t;
        t.table_type = tt;
        t.x_units = ImportUnits::mev;
        t.y_units = tt == ImportTableType::dedx    ? ImportUnits::mev_per_len
                    : tt == ImportTableType::range ? ImportUnits::len
                                                   : tt == ImportTableType::msc_xs ? ImportUnits::mev_sq_per_len : ImportUnits::len_inv;
        for (long m = 0; m < nmat; ++m)
        {
            t.physics_vectors.push_back(
                log_vector(kv, prefix + "." + std::to_string(m)));
        }
        return t;
    };
    auto make_model = [&](std::string const& prefix, ImportModelClass imc) {
        ImportModel model;
        model.model_class = imc;
        for (long m = 0; m < nmat; ++m)
        {
            auto p = prefix + "." + std::to_string(m);
            ImportModelMaterial imm;
            if (kv.has(p + ".energy"))
            {
                imm.energy = kv.dbl(p + ".energy");
                auto nel_mat
                    = kv.dbl("material." + std::to_string(m) + ".elements")
                          .size();
                for (std::size_t e = 0; e < nel_mat; ++e)
                {
                    imm.micro_xs.push_back(
                        kv.dbl(p + ".micro." + std::to_string(e)));
                }
            }
            model.materials.push_back(imm);
        }
        return model;
    };
    auto empty_model = [&](ImportModelClass imc) {
        ImportModel model;
        model.model_class = imc;
        model.materials.resize(nmat);
        return model;
    };

    // Gamma processes
    {
        ImportProcess p;
        p.particle_pdg = 22;
        p.secondary_pdg = 11;
        p.process_type = ImportProcessType::electromagnetic;
        p.process_class = ImportProcessClass::compton;
        p.models.push_back(empty_model(ImportModelClass::klein_nishina));
        p.tables.push_back(
            make_table("table.22.compton.lambda", ImportTableType::lambda));
        data.processes.push_back(p);
    }
    {
        ImportProcess p;
        p.particle_pdg = 22;
        p.secondary_pdg = 11;
        p.process_type = ImportProcessType::electromagnetic;
        p.process_class = ImportProcessClass::photoelectric;
        p.models.push_back(
            empty_model(ImportModelClass::livermore_photoelectric));
        p.tables.push_back(make_table("table.22.photoelectric.lambda",
                                      ImportTableType::lambda));
        data.processes.push_back(p);
    }
    {
        ImportProcess p;
        p.particle_pdg = 22;
        p.secondary_pdg = 11;
        p.process_type = ImportProcessType::electromagnetic;
        p.process_class = ImportProcessClass::conversion;
        p.models.push_back(make_model("model.22.conversion.bethe_heitler",
                                      ImportModelClass::bethe_heitler_lpm));
        p.tables.push_back(
            make_table("table.22.conversion.lambda", ImportTableType::lambda));
        data.processes.push_back(p);
    }
    for (int pdg : {11, -11})
    {
        auto spdg = std::to_string(pdg);
        {
            ImportProcess p;
            p.particle_pdg = pdg;
            p.secondary_pdg = 11;
            p.process_type = ImportProcessType::electromagnetic;
            p.process_class = ImportProcessClass::e_ioni;
            p.models.push_back(empty_model(ImportModelClass::moller_bhabha));
            p.tables.push_back(make_table("table." + spdg + ".e_ioni.lambda",
                                          ImportTableType::lambda));
            p.tables.push_back(make_table("table." + spdg + ".e_ioni.dedx",
                                          ImportTableType::dedx));
            p.tables.push_back(make_table("table." + spdg + ".e_ioni.range",
                                          ImportTableType::range));
            data.processes.push_back(p);
        }
        {
            ImportProcess p;
            p.particle_pdg = pdg;
            p.secondary_pdg = 22;
            p.process_type = ImportProcessType::electromagnetic;
            p.process_class = ImportProcessClass::e_brems;
            p.models.push_back(
                make_model("model." + spdg + ".e_brems.e_brems_sb",
                           ImportModelClass::e_brems_sb));
            p.models.push_back(
                make_model("model." + spdg + ".e_brems.e_brems_lpm",
                           ImportModelClass::e_brems_lpm));
            p.tables.push_back(make_table("table." + spdg + ".e_brems.lambda",
                                          ImportTableType::lambda));
            data.processes.push_back(p);
        }
        if (pdg == -11)
        {
            ImportProcess p;
            p.particle_pdg = pdg;
            p.secondary_pdg = 22;
            p.process_type = ImportProcessType::electromagnetic;
            p.process_class = ImportProcessClass::annihilation;
            p.models.push_back(empty_model(ImportModelClass::e_plus_to_gg));
            data.processes.push_back(p);
        }
        if (with_msc)
        {
            ImportMscModel msc;
            msc.particle_pdg = pdg;
            msc.model_class = ImportModelClass::urban_msc;
            msc.xs_table = make_table("msc." + spdg, ImportTableType::msc_xs);
            data.msc_models.push_back(msc);
        }
    }

    // Seltzer-Berger and Livermore data for each element
    for (auto const& el : data.elements)
    {
        auto z = std::to_string(el.atomic_number);
        ImportSBTable sb;
        sb.x = kv.dbl("sb." + z + ".x");
        sb.y = kv.dbl("sb." + z + ".y");
        sb.value = kv.dbl("sb." + z + ".value");
        data.sb_data[el.atomic_number] = sb;

        ImportLivermorePE pe;
        auto pz = "livermore." + z;
        auto th = kv.dbl(pz + ".thresh");
        pe.thresh_lo = th[0];
        pe.thresh_hi = th[1];
        pe.xs_hi.vector_type = ImportPhysicsVectorType::free;
        pe.xs_hi.x = kv.dbl(pz + ".xs_hi.x");
        pe.xs_hi.y = kv.dbl(pz + ".xs_hi.y");
        if (kv.has(pz + ".xs_lo.x"))
        {
            pe.xs_lo.vector_type = ImportPhysicsVectorType::free;
            pe.xs_lo.x = kv.dbl(pz + ".xs_lo.x");
            pe.xs_lo.y = kv.dbl(pz + ".xs_lo.y");
        }
        long nsh = kv.i(pz + ".shells");
        for (long s = 0; s < nsh; ++s)
        {
            auto ps = pz + ".shell." + std::to_string(s);
            ImportLivermoreSubshell sh;
            sh.binding_energy = kv.d(ps + ".binding");
            sh.param_lo = kv.dbl(ps + ".param_lo");
            sh.param_hi = kv.dbl(ps + ".param_hi");
            sh.energy = kv.dbl(ps + ".energy");
            sh.xs = kv.dbl(ps + ".xs");
            pe.shells.push_back(sh);
        }
        data.livermore_pe_data[el.atomic_number] = pe;
    }

    // Parameters
    data.em_params.energy_loss_fluct = kv.i("em.energy_loss_fluct");
    data.em_params.lpm = kv.i("em.lpm");
    data.em_params.integral_approach = kv.i("em.integral_approach");
    data.em_params.linear_loss_limit = kv.d("em.linear_loss_limit");
    data.em_params.lowest_electron_energy = kv.d("em.lowest_electron_energy");
    data.em_params.msc_range_factor = kv.d("em.msc_range_factor");
    data.em_params.msc_safety_factor = kv.d("em.msc_safety_factor");
    data.em_params.msc_lambda_limit = kv.d("em.msc_lambda_limit");
    {
        auto lp = kv.dbl("trans.looping");
        for (std::size_t j = 0; j + 2 < lp.size() + 0; j += 3)
        {
            ImportLoopingThreshold lt;
            lt.threshold_trials = static_cast<int>(lp[j + 1]);
            lt.important_energy = lp[j + 2];
            data.trans_params.looping[static_cast<int>(lp[j])] = lt;
        }
        data.trans_params.max_substeps = kv.i("trans.max_substeps");
    }
    return data;
}

//---------------------------------------------------------------------------//
// Geometry: ORANGE through orangeinp
//---------------------------------------------------------------------------//
using namespace celeritas::orangeinp;

SPConstObject make_box(std::string label, Real3 const& lo, Real3 const& hi)
{
    Real3 half{(hi[0] - lo[0]) / 2, (hi[1] - lo[1]) / 2, (hi[2] - lo[2]) / 2};
    Real3 center{(hi[0] + lo[0]) / 2, (hi[1] + lo[1]) / 2, (hi[2] + lo[2]) / 2};
    SPConstObject result
        = std::make_shared<BoxShape>(std::move(label), Box{half});
    if (center[0] != 0 || center[1] != 0 || center[2] != 0)
    {
        result = std::make_shared<Transformed>(std::move(result),
                                               Translation{center});
    }
    return result;
}

struct GeoSpec
{
    std::shared_ptr<OrangeParams> geo;
    std::vector<std::string> vol_labels;  // tally volume labels
    std::map<std::string, MaterialId> label_to_mat;
};

//! Sampling calorimeter: 50 x (2.3 mm Pb + 5.7 mm lAr), 40x40 cm, along +z,
//! front face at z = 0, in a vacuum world box of half-width 30 cm in x/y and
//! spanning z in [-10, 50].
GeoSpec build_calo()
{
    constexpr int num_layers = 50;
    constexpr double pb = 0.23, lar = 0.57, pitch = pb + lar;
    constexpr double half_xy = 20.0;

    UnitProto::Input inp;
    inp.label = "calo";
    inp.boundary.interior
        = make_box("world", {-30, -30, -10}, {30, 30, 50});
    inp.boundary.zorder = ZOrder::exterior;
    inp.background.fill = GeoMaterialId{0};
    inp.background.label = Label{"world"};

    GeoSpec spec;
    spec.label_to_mat["world"] = MaterialId{0};
    for (int k = 0; k < num_layers; ++k)
    {
        double z0 = k * pitch;
        double z1 = z0 + pb;
        double z2 = (k + 1) * pitch;
        auto pbl = "pb_" + std::to_string(k);
        auto arl = "lar_" + std::to_string(k);
        inp.materials.push_back({make_box(pbl, {-half_xy, -half_xy, z0},
                                          {half_xy, half_xy, z1}),
                                 GeoMaterialId{1},
                                 Label{pbl}});
        inp.materials.push_back({make_box(arl, {-half_xy, -half_xy, z1},
                                          {half_xy, half_xy, z2}),
                                 GeoMaterialId{2},
                                 Label{arl}});
        spec.label_to_mat[pbl] = MaterialId{1};
        spec.label_to_mat[arl] = MaterialId{2};
        spec.vol_labels.push_back(pbl);
        spec.vol_labels.push_back(arl);
    }

    InputBuilder::Options opts;
    opts.tol = Tolerance<>::from_default();
    InputBuilder build(std::move(opts));
    UnitProto global(std::move(inp));
    spec.geo = std::make_shared<OrangeParams>(build(global));
    return spec;
}

//! CMS-like detector of concentric shells about z (the GB300 build's
//! make_cms_geometry): 10 Si layers of 0.3 mm with inner radii evenly from 4
//! to 110 cm (|z| < 270), a PbWO4 barrel (129-152 cm, |z| < 300) and 17 brass
//! (5 cm) + scintillator (0.4 cm) pairs from 180 cm with pitch 115/17 cm
//! (|z| < 300), in a vacuum world box 620 x 620 x 640 cm.
GeoSpec build_cms()
{
    UnitProto::Input inp;
    inp.label = "cms";
    inp.boundary.interior = make_box("world", {-310, -310, -320}, {310, 310, 320});
    inp.boundary.zorder = ZOrder::exterior;
    inp.background.fill = GeoMaterialId{0};
    inp.background.label = Label{"world"};

    GeoSpec spec;
    spec.label_to_mat["world"] = MaterialId{0};
    auto add_shell = [&](std::string const& label,
                         double r_in,
                         double r_out,
                         double hz,
                         int mat) {
        auto shell = std::make_shared<CylinderSolid>(
            std::string(label), Cylinder{r_out, hz}, Cylinder{r_in, hz});
        inp.materials.push_back(
            {std::move(shell), GeoMaterialId{static_cast<size_type>(mat)}, Label{label}});
        spec.label_to_mat[label] = MaterialId{static_cast<size_type>(mat)};
        spec.vol_labels.push_back(label);
    };
    for (int k = 0; k < 10; ++k)
    {
        double r = 4.0 + k * (110.0 - 4.0) / 9;
        add_shell("si_" + std::to_string(k), r, r + 0.03, 270, 1);
    }
    add_shell("ecal", 129, 152, 300, 2);
    double const pitch = (295.0 - 180.0) / 17;
    for (int k = 0; k < 17; ++k)
    {
        double r = 180.0 + k * pitch;
        add_shell("brass_" + std::to_string(k), r, r + 5.0, 300, 3);
        add_shell("scint_" + std::to_string(k), r + 5.0, r + 5.4, 300, 4);
    }

    InputBuilder::Options opts;
    opts.tol = Tolerance<>::from_default();
    InputBuilder build(std::move(opts));
    UnitProto global(std::move(inp));
    spec.geo = std::make_shared<OrangeParams>(build(global));
    return spec;
}

//! Geometry from the GB300 build's geometry file format ('gbx-geometry 1';
//! world, background, box and shell records): boxes as BoxShape objects,
//! shells as CylinderSolid objects translated along z when not centred
GeoSpec build_from_file(std::string const& path)
{
    std::ifstream in(path);
    CELER_VALIDATE(in, << "cannot open geometry file " << path);
    UnitProto::Input inp;
    inp.label = "file";
    inp.boundary.zorder = ZOrder::exterior;
    inp.background.label = Label{"world"};
    inp.background.fill = GeoMaterialId{0};
    GeoSpec spec;
    spec.label_to_mat["world"] = MaterialId{0};
    std::string line;
    while (std::getline(in, line))
    {
        auto hash = line.find('#');
        if (hash != std::string::npos)
            line.erase(hash);
        std::istringstream ls(line);
        std::string kind;
        if (!(ls >> kind) || kind == "gbx-geometry")
            continue;
        if (kind == "world")
        {
            Real3 lo, hi;
            ls >> lo[0] >> lo[1] >> lo[2] >> hi[0] >> hi[1] >> hi[2];
            inp.boundary.interior = make_box("world", lo, hi);
        }
        else if (kind == "background")
        {
            size_type m;
            ls >> m;
            inp.background.fill = GeoMaterialId{m};
            spec.label_to_mat["world"] = MaterialId{m};
        }
        else if (kind == "box" || kind == "shell")
        {
            std::string label;
            size_type m;
            ls >> label >> m;
            SPConstObject obj;
            if (kind == "box")
            {
                Real3 lo, hi;
                ls >> lo[0] >> lo[1] >> lo[2] >> hi[0] >> hi[1] >> hi[2];
                obj = make_box(label, lo, hi);
            }
            else
            {
                double r_in, r_out, z_lo, z_hi;
                ls >> r_in >> r_out >> z_lo >> z_hi;
                double hz = (z_hi - z_lo) / 2, zc = (z_hi + z_lo) / 2;
                obj = std::make_shared<CylinderSolid>(
                    std::string(label), Cylinder{r_out, hz}, Cylinder{r_in, hz});
                if (zc != 0)
                {
                    obj = std::make_shared<Transformed>(std::move(obj),
                                                        Translation{Real3{0, 0, zc}});
                }
            }
            CELER_VALIDATE(ls, << "bad record in " << path << ": " << line);
            inp.materials.push_back({std::move(obj), GeoMaterialId{m}, Label{label}});
            spec.label_to_mat[label] = MaterialId{m};
            spec.vol_labels.push_back(label);
        }
        else
        {
            CELER_VALIDATE(false, << "unknown record in " << path << ": " << kind);
        }
    }
    InputBuilder::Options opts;
    opts.tol = Tolerance<>::from_default();
    InputBuilder build(std::move(opts));
    UnitProto global(std::move(inp));
    spec.geo = std::make_shared<OrangeParams>(build(global));
    return spec;
}

GeoSpec build_geometry(std::string const& name)
{
    if (name == "calo")
        return build_calo();
    if (name == "cms")
        return build_cms();
    return build_from_file(name);
}

//---------------------------------------------------------------------------//
// Problem construction (mirrors Runner::build_core_params)
//---------------------------------------------------------------------------//
//---------------------------------------------------------------------------//
// Hit printer: a step interface over SimpleCalo's detector volumes (same
// volume -> detector map, steps without deposition dropped) that gathers
// every step datum, copies each step's hits with the reference's own
// copy_steps and prints them; it also sums the deposition per detector so
// that the run still prints its 'edep' lines
//---------------------------------------------------------------------------//
class HitPrinter final : public StepInterface
{
  public:
    HitPrinter(Filters filters, size_type num_detectors)
        : filters_(std::move(filters)), edep_(num_detectors, 0.0)
    {
    }

    Filters filters() const final { return filters_; }
    StepSelection selection() const final { return StepSelection::all(); }

    void process_steps(HostStepState state) final
    {
        DetectorStepOutput out;
        copy_steps<MemSpace::host>(&out, state.steps);
        auto const& pre = out.points[StepPoint::pre];
        auto const& post = out.points[StepPoint::post];
        for (size_type i = 0; i < out.size(); ++i)
        {
            std::printf(
                "hit %u %u %u %u %u %u %u %.17g %.17g %.17g %.17g %.17g %.17g "
                "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g "
                "%.17g %.17g\n",
                step_,
                out.detector[i].unchecked_get(),
                out.track_id[i].unchecked_get(),
                out.event_id[i].unchecked_get(),
                out.parent_id[i].unchecked_get(),
                out.track_step_count[i],
                out.particle[i].unchecked_get(),
                out.step_length[i],
                out.energy_deposition[i].value(),
                pre.time[i],
                pre.pos[i][0],
                pre.pos[i][1],
                pre.pos[i][2],
                pre.dir[i][0],
                pre.dir[i][1],
                pre.dir[i][2],
                pre.energy[i].value(),
                post.time[i],
                post.pos[i][0],
                post.pos[i][1],
                post.pos[i][2],
                post.dir[i][0],
                post.dir[i][1],
                post.dir[i][2],
                post.energy[i].value());
            edep_[out.detector[i].unchecked_get()]
                += out.energy_deposition[i].value();
        }
        ++step_;
    }
    void process_steps(DeviceStepState) final
    {
        throw std::runtime_error("host-only hit printer");
    }

    std::vector<double> const& edep() const { return edep_; }

  private:
    Filters filters_;
    std::vector<double> edep_;
    unsigned int step_{0};
};

//! R-Z field map from the text form shared with the GB300 build: header
//! 'rzmap num_z num_r min_z max_z min_r max_r' [cm], then 'Bz Br' [tesla]
//! per node, [z][r]; converted to native units as the reference's inputs are
RZMapFieldInput load_rzmap(std::string const& path)
{
    std::ifstream in(path);
    CELER_VALIDATE(in, << "cannot open field map " << path);
    std::string tag;
    RZMapFieldInput inp;
    in >> tag >> inp.num_grid_z >> inp.num_grid_r >> inp.min_z >> inp.max_z
        >> inp.min_r >> inp.max_r;
    CELER_VALIDATE(in && tag == "rzmap", << "bad field map header");
    std::size_t const n = std::size_t(inp.num_grid_z) * inp.num_grid_r;
    inp.field_z.resize(n);
    inp.field_r.resize(n);
    for (std::size_t i = 0; i < n; ++i)
    {
        double bz, br;
        in >> bz >> br;
        inp.field_z[i] = native_value_from(units::FieldTesla{bz});
        inp.field_r[i] = native_value_from(units::FieldTesla{br});
    }
    CELER_VALIDATE(in, << "truncated field map");
    return inp;
}

//! Set one FieldDriverOptions member by name (celer-sim's field_options)
void set_field_option(FieldDriverOptions* o, std::string const& name, double v)
{
#define GBX_FIELD_OPTION(M)                    \
    if (name == #M)                            \
    {                                          \
        o->M = static_cast<decltype(o->M)>(v); \
        return;                                \
    }
    GBX_FIELD_OPTION(minimum_step)
    GBX_FIELD_OPTION(delta_chord)
    GBX_FIELD_OPTION(delta_intersection)
    GBX_FIELD_OPTION(epsilon_step)
    GBX_FIELD_OPTION(epsilon_rel_max)
    GBX_FIELD_OPTION(errcon)
    GBX_FIELD_OPTION(pgrow)
    GBX_FIELD_OPTION(pshrink)
    GBX_FIELD_OPTION(safety)
    GBX_FIELD_OPTION(max_stepping_increase)
    GBX_FIELD_OPTION(max_stepping_decrease)
    GBX_FIELD_OPTION(max_nsteps)
    GBX_FIELD_OPTION(max_substeps)
#undef GBX_FIELD_OPTION
    throw std::runtime_error("unknown field option " + name);
}

struct Problem
{
    std::shared_ptr<CoreParams> core;
    std::shared_ptr<SimpleCalo> calo;
    std::shared_ptr<HitPrinter> hits;
    std::shared_ptr<StepCollector> collector;
    GeoSpec geo;
};

Problem build_problem(ImportData const& imported,
                      std::string const& geo_name,
                      unsigned int seed,
                      Real3 field,
                      bool msc,
                      TrackOrder track_order,
                      bool print_hits,
                      std::string const& rz_field,
                      size_type num_streams = 1,
                      bool brem_combined = false,
                      FieldDriverOptions const& driver_options = {})
{
    Problem prob;
    prob.geo = build_geometry(geo_name);

    CoreParams::Input params;
    params.action_reg = std::make_shared<ActionRegistry>();
    params.output_reg = std::make_shared<OutputRegistry>();
    params.geometry = prob.geo.geo;
    params.material = MaterialParams::from_import(imported);
    {
        GeoMaterialParams::Input gm;
        gm.geometry = params.geometry;
        gm.materials = params.material;
        auto const& vols = params.geometry->volumes();
        for (auto vid : range(VolumeId{vols.size()}))
        {
            auto const& lab = vols.at(vid);
            auto it = prob.geo.label_to_mat.find(lab.name);
            gm.volume_to_mat.push_back(
                it == prob.geo.label_to_mat.end() ? MaterialId{} : it->second);
        }
        params.geomaterial
            = std::make_shared<GeoMaterialParams>(std::move(gm));
    }
    params.particle = ParticleParams::from_import(imported);
    params.cutoff = CutoffParams::from_import(
        imported, params.particle, params.material);

    params.physics = [&] {
        PhysicsParams::Input input;
        input.particles = params.particle;
        input.materials = params.material;
        input.action_registry = params.action_reg.get();
        input.options.secondary_stack_factor = 3;
        input.options.linear_loss_limit = imported.em_params.linear_loss_limit;
        input.options.lowest_electron_energy = PhysicsParamsOptions::Energy(
            imported.em_params.lowest_electron_energy);
        ProcessBuilder::Options opts;
        // RunnerInput::brem_combined (app/celer-sim/RunnerInput.hh:120)
        opts.brem_combined = brem_combined;
        opts.brems_selection = BremsModelSelection::all;
        ProcessBuilder build_process(
            imported, params.particle, params.material, opts);
        for (auto p :
             ProcessBuilder::get_all_process_classes(imported.processes))
        {
            input.processes.push_back(build_process(p));
        }
        return std::make_shared<PhysicsParams>(std::move(input));
    }();

    bool eloss = imported.em_params.energy_loss_fluct;
    auto urban = msc ? UrbanMscParams::from_import(
                           *params.particle, *params.material, imported)
                     : nullptr;
    if (!rz_field.empty())
    {
        auto along_step = AlongStepRZMapFieldMscAction::from_params(
            params.action_reg->next_id(),
            *params.material,
            *params.particle,
            [&] {
                auto inp = load_rzmap(rz_field);
                inp.driver_options = driver_options;
                return inp;
            }(),
            urban,
            eloss);
        params.action_reg->insert(along_step);
    }
    else if (field[0] == 0 && field[1] == 0 && field[2] == 0)
    {
        auto along_step = AlongStepGeneralLinearAction::from_params(
            params.action_reg->next_id(),
            *params.material,
            *params.particle,
            urban,
            eloss);
        params.action_reg->insert(along_step);
    }
    else
    {
        UniformFieldParams field_params;
        field_params.field = field;
        field_params.options = driver_options;
        for (real_type& v : field_params.field)
        {
            v = native_value_from(units::FieldTesla{v});
        }
        auto along_step = AlongStepUniformMscAction::from_params(
            params.action_reg->next_id(),
            *params.material,
            *params.particle,
            field_params,
            urban,
            eloss);
        params.action_reg->insert(along_step);
    }
    params.rng = std::make_shared<RngParams>(seed);
    params.sim = SimParams::from_import(
        imported, params.particle, FieldDriverOptions{}.max_substeps);
    params.max_streams = num_streams;
    {
        TrackInitParams::Input input;
        input.capacity = 1u << 22;
        input.max_events = 1u << 16;
        input.track_order = track_order;
        params.init = std::make_shared<TrackInitParams>(input);
    }

    prob.core = std::make_shared<CoreParams>(std::move(params));

    // Energy deposition tally over the listed volumes
    {
        std::vector<Label> labels;
        for (auto const& l : prob.geo.vol_labels)
            labels.push_back(Label{l});
        prob.calo = std::make_shared<SimpleCalo>(
            std::move(labels), *prob.core->geometry(), num_streams);
        StepCollector::VecInterface ifaces{prob.calo};
        if (print_hits)
        {
            // The printer takes the calorimeter's volumes (one step
            // interface per volume): same registered actions
            prob.hits = std::make_shared<HitPrinter>(prob.calo->filters(),
                                                     prob.calo->num_detectors());
            ifaces = {prob.hits};
        }
        prob.collector = std::make_shared<StepCollector>(
            prob.core->geometry(),
            std::move(ifaces),
            prob.core->aux_reg().get(),
            prob.core->action_reg().get());
    }
    return prob;
}

//---------------------------------------------------------------------------//
// Primaries file: "pdg energy x y z dx dy dz time event" per line
//---------------------------------------------------------------------------//
std::vector<Primary>
load_primaries(std::string const& path, ParticleParams const& particles)
{
    std::ifstream in(path);
    if (!in)
        throw std::runtime_error("cannot open " + path);
    std::vector<Primary> result;
    int pdg;
    double e, x, y, z, dx, dy, dz, t;
    long ev;
    while (in >> pdg >> e >> x >> y >> z >> dx >> dy >> dz >> t >> ev)
    {
        Primary p;
        p.particle_id = particles.find(PDGNumber{pdg});
        p.energy = units::MevEnergy{e};
        p.position = {x, y, z};
        p.direction = {dx, dy, dz};
        p.time = t;
        p.event_id = EventId{static_cast<size_type>(ev)};
        result.push_back(p);
    }
    return result;
}

//! Print every non-inactive track slot (same fields as the port's trace)
void trace_state(Stepper<MemSpace::host>& step, CoreParams const& core, size_type iter)
{
    auto const& st
        = dynamic_cast<CoreState<MemSpace::host> const&>(step.state());
    auto const& pref = core.ref<MemSpace::host>();
    auto const& sref = st.ref();
    for (size_type i = 0; i < st.size(); ++i)
    {
        CoreTrackView track(pref, sref, TrackSlotId{i});
        auto sim = track.make_sim_view();
        if (sim.status() == TrackStatus::inactive)
            continue;
        auto par = track.make_particle_view();
        auto geo = track.make_geo_view();
        auto phys = track.make_physics_view();
        auto pstep = track.make_physics_step_view();
        auto const& pos = geo.pos();
        auto const& dir = geo.dir();
        std::printf("trace %u %u st=%d pid=%u E=%.17g pos=(%.17g,%.17g,%.17g) "
                    "dir=(%.17g,%.17g,%.17g) vol=%u act=%d len=%.17g mfp=%.17g "
                    "edep=%.17g nsec=%u\n",
                    iter,
                    i,
                    static_cast<int>(sim.status()),
                    par.particle_id().unchecked_get(),
                    par.energy().value(),
                    pos[0], pos[1], pos[2], dir[0], dir[1], dir[2],
                    geo.is_outside() ? 0u : geo.volume_id().unchecked_get(),
                    static_cast<int>(sim.post_step_action().unchecked_get()),
                    sim.step_length(),
                    phys.interaction_mfp(),
                    pstep.energy_deposition().value(),
                    static_cast<unsigned>(pstep.secondaries().size()));
    }
}

int run(int argc, char** argv)
{
    if (argc < 7)
    {
        std::cerr << "usage: run <physics> <geometry> <primaries> <slots> "
                     "<seed> [--field Bx By Bz] [--msc] [--steps N] "
                     "[--track-order N] [--reseed EVENT] [--dump-rng N] [--hits] "
                     "[--rz-field FILE] [--brem-combined]\n";
        return 2;
    }
    std::string phys_path = argv[2], geo_name = argv[3], prim_path = argv[4];
    size_type num_slots = std::stoul(argv[5]);
    unsigned int seed = std::stoul(argv[6]);
    Real3 field{0, 0, 0};
    bool msc = false;
    size_type max_steps = static_cast<size_type>(-1);
    TrackOrder track_order = TrackOrder::none;
    bool trace = false;
    long long reseed = -1;
    size_type dump_rng = 0;
    bool print_hits = false;
    bool brem_combined = false;
    FieldDriverOptions driver_options;
    std::string rz_field;
    for (int i = 7; i < argc; ++i)
    {
        std::string a = argv[i];
        if (a == "--field")
        {
            field = {std::strtod(argv[i + 1], nullptr),
                     std::strtod(argv[i + 2], nullptr),
                     std::strtod(argv[i + 3], nullptr)};
            i += 3;
        }
        else if (a == "--msc")
            msc = true;
        else if (a == "--steps")
            max_steps = std::stoul(argv[++i]);
        else if (a == "--track-order")
            track_order = static_cast<TrackOrder>(std::stoi(argv[++i]));
        else if (a == "--trace")
            trace = true;
        else if (a == "--reseed")
            reseed = std::stoull(argv[++i]);
        else if (a == "--dump-rng")
            dump_rng = std::stoul(argv[++i]);
        else if (a == "--hits")
            print_hits = true;
        else if (a == "--rz-field")
            rz_field = argv[++i];
        else if (a == "--brem-combined")
            brem_combined = true;
        else if (a == "--field-option" && i + 2 < argc)
        {
            set_field_option(&driver_options, argv[i + 1], std::strtod(argv[i + 2], nullptr));
            i += 2;
        }
    }
    CELER_VALIDATE(driver_options, << "invalid field driver options");

    KvFile kv(phys_path);
    ImportData imported = load_import(kv, msc);
    Problem prob = build_problem(imported,
                                 geo_name,
                                 seed,
                                 field,
                                 msc,
                                 track_order,
                                 print_hits,
                                 rz_field,
                                 1,
                                 brem_combined,
                                 driver_options);
    auto primaries = load_primaries(prim_path, *prob.core->particle());

    StepperInput sinp;
    sinp.params = prob.core;
    sinp.stream_id = StreamId{0};
    sinp.num_track_slots = num_slots;
    Stepper<MemSpace::host> step(std::move(sinp));
    if (reseed >= 0)
    {
        // Stepper::reseed before the event, as accel::LocalTransporter does
        step.reseed(UniqueEventId(static_cast<UniqueEventId::size_type>(reseed)));
    }
    for (size_type i = 0; i < std::min<size_type>(dump_rng, num_slots); ++i)
    {
        auto const& r = step.state_ref().rng.state[TrackSlotId{i}];
        std::printf("rng %u %u %u %u %u %u %u\n",
                    i,
                    r.xorstate[0],
                    r.xorstate[1],
                    r.xorstate[2],
                    r.xorstate[3],
                    r.xorstate[4],
                    r.weylstate);
    }

    // Print action list (ordered) for the action-ID contract
    {
        auto const& reg = *prob.core->action_reg();
        for (auto id : range(ActionId{reg.num_actions()}))
        {
            std::printf("action %u %s\n",
                        id.unchecked_get(),
                        std::string(reg.id_to_label(id)).c_str());
        }
    }

    StepperResult counts = step(make_span(primaries));
    size_type iter = 0;
    if (trace)
        trace_state(step, *prob.core, iter);
    unsigned long long track_steps = counts.active;
    std::printf("step %u %u %u %u %u\n",
                iter,
                counts.generated,
                counts.queued,
                counts.active,
                counts.alive);
    while (counts && ++iter < max_steps)
    {
        counts = step();
        if (trace)
            trace_state(step, *prob.core, iter);
        track_steps += counts.active;
        std::printf("step %u %u %u %u %u\n",
                    iter,
                    counts.generated,
                    counts.queued,
                    counts.active,
                    counts.alive);
    }
    std::printf("total_steps %llu iterations %u\n", track_steps, iter + 1);
    auto edep = prob.hits ? prob.hits->edep()
                          : prob.calo->calc_total_energy_deposition();
    for (std::size_t i = 0; i < edep.size(); ++i)
    {
        std::printf("edep %s %.17g\n", prob.geo.vol_labels[i].c_str(), edep[i]);
    }
    return 0;
}

//! One interaction per input, through the reference's own model actions.
//! Each input line (model label, PDG, energy [MeV], position [cm],
//! direction, element component) becomes a primary of its own event. The
//! step actions up to and including pre-step (extend-from-primaries,
//! initialize-tracks, pre-step: ActionSequence.cc:77-138) prepare the tracks
//! as in a step; then each track's step-limit action and element component
//! are set as physics-discrete-select would (PhysicsStepUtils.hh:253-308)
//! and only the named models run (their InteractionApplier executors).
//! Prints per input the track after the interaction, its random state and
//! its secondaries.
int interact(int argc, char** argv)
{
    if (argc < 6)
    {
        std::cerr << "usage: interact <physics> <geometry> <inputs> <seed> "
                     "[--msc] [--brem-combined]\n";
        return 2;
    }
    std::string phys_path = argv[2], geo_name = argv[3], in_path = argv[4];
    unsigned int seed = std::stoul(argv[5]);
    bool msc = false;
    bool brem_combined = false;
    for (int i = 6; i < argc; ++i)
    {
        std::string a = argv[i];
        if (a == "--msc")
            msc = true;
        else if (a == "--brem-combined")
            brem_combined = true;
    }
    KvFile kv(phys_path);
    ImportData imported = load_import(kv, msc);
    Problem prob = build_problem(imported,
                                 geo_name,
                                 seed,
                                 Real3{0, 0, 0},
                                 msc,
                                 TrackOrder::none,
                                 false,
                                 "",
                                 1,
                                 brem_combined);
    CoreParams const& core = *prob.core;
    ParticleParams const& particles = *core.particle();

    std::ifstream in(in_path);
    CELER_VALIDATE(in, << "cannot open " << in_path);
    std::vector<Primary> primaries;
    std::vector<std::string> models;
    std::vector<unsigned int> elcomps;
    std::string model;
    int pdg;
    double e, x, y, z, dx, dy, dz;
    unsigned int elcomp;
    while (in >> model >> pdg >> e >> x >> y >> z >> dx >> dy >> dz >> elcomp)
    {
        Primary p;
        p.particle_id = particles.find(PDGNumber{pdg});
        CELER_VALIDATE(p.particle_id, << "unknown PDG " << pdg);
        p.energy = units::MevEnergy{e};
        p.position = {x, y, z};
        p.direction = {dx, dy, dz};
        p.time = 0;
        p.event_id = EventId{static_cast<size_type>(primaries.size())};
        primaries.push_back(p);
        models.push_back(model);
        elcomps.push_back(elcomp);
    }
    CELER_VALIDATE(!primaries.empty(), << "no inputs in " << in_path);

    StepperInput sinp;
    sinp.params = prob.core;
    sinp.stream_id = StreamId{0};
    sinp.num_track_slots = static_cast<size_type>(primaries.size());
    Stepper<MemSpace::host> step(std::move(sinp));
    auto& state = dynamic_cast<CoreState<MemSpace::host>&>(*step.sp_state());
    ExtendFromPrimariesAction::find_action(core)->insert(
        core, state, make_span(primaries));
    state.counters().num_generated = 0;
    for (auto const& action : step.actions().actions().step())
    {
        if (action->order() > StepActionOrder::pre)
            break;
        action->step(core, state);
    }

    auto const& reg = *core.action_reg();
    auto const& pref = core.ref<MemSpace::host>();
    auto const& sref = state.ref();
    // The pre-step's results per input: step limit and its action, sampled
    // interaction MFP, macroscopic and per-process cross sections, range
    for (size_type i = 0; i < state.size(); ++i)
    {
        CoreTrackView track(pref, sref, TrackSlotId{i});
        auto sim = track.make_sim_view();
        auto phys = track.make_physics_view();
        auto pstep = track.make_physics_step_view();
        std::printf("pre %u act=%u len=%.17g mfp=%.17g macro=%.17g range=%.17g xs=",
                    sim.event_id().unchecked_get(),
                    sim.post_step_action().unchecked_get(),
                    sim.step_length(),
                    phys.interaction_mfp(),
                    pstep.macro_xs(),
                    phys.dedx_range());
        for (auto ppid : range(ParticleProcessId{phys.num_particle_processes()}))
        {
            std::printf("%s%.17g", ppid.get() ? "," : "", pstep.per_process_xs(ppid));
        }
        std::printf("\n");
    }
    std::vector<ActionId> to_run;
    for (size_type i = 0; i < state.size(); ++i)
    {
        CoreTrackView track(pref, sref, TrackSlotId{i});
        auto sim = track.make_sim_view();
        CELER_VALIDATE(sim.status() == TrackStatus::alive,
                       << "track slot " << i << " is not alive after pre-step");
        size_type const idx = sim.event_id().unchecked_get();
        ActionId aid = reg.find_action(models[idx]);
        CELER_VALIDATE(aid, << "no action '" << models[idx] << "'");
        sim.post_step_action(aid);
        track.make_physics_step_view().element(ElementComponentId{elcomps[idx]});
        if (std::find(to_run.begin(), to_run.end(), aid) == to_run.end())
            to_run.push_back(aid);
    }
    std::sort(to_run.begin(), to_run.end());
    for (ActionId aid : to_run)
    {
        auto const* action
            = dynamic_cast<CoreStepActionInterface const*>(reg.action(aid).get());
        CELER_VALIDATE(action, << "action " << aid.unchecked_get() << " does not step");
        action->step(core, state);
    }

    std::vector<size_type> slot_of(primaries.size());
    for (size_type i = 0; i < state.size(); ++i)
    {
        CoreTrackView track(pref, sref, TrackSlotId{i});
        slot_of[track.make_sim_view().event_id().unchecked_get()] = i;
    }
    for (size_type idx = 0; idx < slot_of.size(); ++idx)
    {
        size_type const i = slot_of[idx];
        CoreTrackView track(pref, sref, TrackSlotId{i});
        auto sim = track.make_sim_view();
        auto par = track.make_particle_view();
        auto geo = track.make_geo_view();
        auto pstep = track.make_physics_step_view();
        auto const& dir = geo.dir();
        auto const& r = sref.rng.state[TrackSlotId{i}];
        auto secondaries = pstep.secondaries();
        std::printf("int %u %s st=%d act=%u mat=%u E=%.17g dir=(%.17g,%.17g,%.17g) "
                    "edep=%.17g nsec=%u rng=%u,%u,%u,%u,%u,%u\n",
                    idx,
                    models[idx].c_str(),
                    static_cast<int>(sim.status()),
                    sim.post_step_action().unchecked_get(),
                    track.make_material_view().material_id().unchecked_get(),
                    par.energy().value(),
                    dir[0], dir[1], dir[2],
                    pstep.energy_deposition().value(),
                    static_cast<unsigned>(secondaries.size()),
                    r.xorstate[0], r.xorstate[1], r.xorstate[2],
                    r.xorstate[3], r.xorstate[4], r.weylstate);
        for (size_type k = 0; k < secondaries.size(); ++k)
        {
            Secondary const& sec = secondaries[k];
            std::printf("sec %u %u pdg=%d E=%.17g dir=(%.17g,%.17g,%.17g)\n",
                        idx,
                        k,
                        sec ? particles.id_to_pdg(sec.particle_id).get() : 0,
                        sec.energy.value(),
                        sec.direction[0], sec.direction[1], sec.direction[2]);
        }
    }
    return 0;
}

//! One along-step per input, through the reference's own actions: each input
//! line (as for 'interact'; the label is not used) becomes a primary of its
//! own event, and the step actions up to and including the along-step ones
//! run (ActionSequence.cc:77-138), then physics-discrete-select. Prints per
//! input the step limit's action, the action after discrete selection and
//! the element component it chose, the step length, position, direction,
//! energy, local deposition, status and random state.
int along(int argc, char** argv)
{
    if (argc < 6)
    {
        std::cerr << "usage: along <physics> <geometry> <inputs> <seed> "
                     "[--field Bx By Bz] [--msc]\n";
        return 2;
    }
    std::string phys_path = argv[2], geo_name = argv[3], in_path = argv[4];
    unsigned int seed = std::stoul(argv[5]);
    Real3 field{0, 0, 0};
    bool msc = false;
    for (int i = 6; i < argc; ++i)
    {
        std::string a = argv[i];
        if (a == "--msc")
            msc = true;
        else if (a == "--field" && i + 3 < argc)
        {
            field = {std::strtod(argv[i + 1], nullptr),
                     std::strtod(argv[i + 2], nullptr),
                     std::strtod(argv[i + 3], nullptr)};
            i += 3;
        }
    }
    KvFile kv(phys_path);
    ImportData imported = load_import(kv, msc);
    Problem prob = build_problem(
        imported, geo_name, seed, field, msc, TrackOrder::none, false, "", 1);
    CoreParams const& core = *prob.core;
    ParticleParams const& particles = *core.particle();

    std::ifstream in(in_path);
    CELER_VALIDATE(in, << "cannot open " << in_path);
    std::vector<Primary> primaries;
    std::string label;
    int pdg;
    double e, x, y, z, dx, dy, dz;
    unsigned int elcomp;
    while (in >> label >> pdg >> e >> x >> y >> z >> dx >> dy >> dz >> elcomp)
    {
        Primary p;
        p.particle_id = particles.find(PDGNumber{pdg});
        CELER_VALIDATE(p.particle_id, << "unknown PDG " << pdg);
        p.energy = units::MevEnergy{e};
        p.position = {x, y, z};
        p.direction = {dx, dy, dz};
        p.time = 0;
        p.event_id = EventId{static_cast<size_type>(primaries.size())};
        primaries.push_back(p);
    }
    CELER_VALIDATE(!primaries.empty(), << "no inputs in " << in_path);

    StepperInput sinp;
    sinp.params = prob.core;
    sinp.stream_id = StreamId{0};
    sinp.num_track_slots = static_cast<size_type>(primaries.size());
    Stepper<MemSpace::host> step(std::move(sinp));
    auto& state = dynamic_cast<CoreState<MemSpace::host>&>(*step.sp_state());
    ExtendFromPrimariesAction::find_action(core)->insert(
        core, state, make_span(primaries));
    state.counters().num_generated = 0;
    auto const& pref = core.ref<MemSpace::host>();
    auto const& sref = state.ref();
    std::vector<ActionId> along_action(state.size());
    bool selected = false;
    for (auto const& action : step.actions().actions().step())
    {
        if (action->order() > StepActionOrder::pre_post)
            break;
        if (action->order() > StepActionOrder::along && !selected)
        {
            // Step limits of the along-step, before discrete selection
            for (size_type i = 0; i < state.size(); ++i)
            {
                CoreTrackView track(pref, sref, TrackSlotId{i});
                along_action[i] = track.make_sim_view().post_step_action();
            }
            selected = true;
        }
        action->step(core, state);
    }
    ActionId const rejected
        = core.action_reg()->find_action("physics-integral-rejected");

    std::vector<size_type> slot_of(primaries.size());
    for (size_type i = 0; i < state.size(); ++i)
    {
        CoreTrackView track(pref, sref, TrackSlotId{i});
        slot_of[track.make_sim_view().event_id().unchecked_get()] = i;
    }
    for (size_type idx = 0; idx < slot_of.size(); ++idx)
    {
        size_type const i = slot_of[idx];
        CoreTrackView track(pref, sref, TrackSlotId{i});
        auto sim = track.make_sim_view();
        auto par = track.make_particle_view();
        auto geo = track.make_geo_view();
        auto pstep = track.make_physics_step_view();
        auto const& pos = geo.pos();
        auto const& dir = geo.dir();
        auto const& r = sref.rng.state[TrackSlotId{i}];
        // A discrete interaction was selected: its element component
        ActionId const sel = sim.post_step_action();
        int const el = (sel != along_action[i] && sel != rejected)
                           ? static_cast<int>(pstep.element().unchecked_get())
                           : -1;
        std::printf("along %u st=%d act=%u sel=%u el=%d len=%.17g "
                    "pos=(%.17g,%.17g,%.17g) "
                    "dir=(%.17g,%.17g,%.17g) E=%.17g edep=%.17g "
                    "rng=%u,%u,%u,%u,%u,%u\n",
                    idx,
                    static_cast<int>(sim.status()),
                    along_action[i].unchecked_get(),
                    sel.unchecked_get(),
                    el,
                    sim.step_length(),
                    pos[0], pos[1], pos[2], dir[0], dir[1], dir[2],
                    par.energy().value(),
                    pstep.energy_deposition().value(),
                    r.xorstate[0], r.xorstate[1], r.xorstate[2],
                    r.xorstate[3], r.xorstate[4], r.weylstate);
    }
    return 0;
}

//! Timed CPU run of the reference's host stepper: events distributed over
//! threads, one Stepper<host> per thread on its own stream, each event
//! transported to completion (celer-sim with CELERITAS_OPENMP=event,
//! app/celer-sim/celer-sim.cc:126-138). A per-event step cap stands in for
//! celer-sim's max_steps (an event that reaches it is counted as capped).
int bench(int argc, char** argv)
{
    if (argc < 7)
    {
        std::cerr << "usage: bench <physics> <geometry> <primaries> <slots> "
                     "<seed> [--threads T] [--field Bx By Bz] [--msc] "
                     "[--rz-field FILE] [--max-steps N]\n";
        return 2;
    }
    std::string phys_path = argv[2], geo_name = argv[3], prim_path = argv[4];
    size_type num_slots = std::stoul(argv[5]);
    unsigned int seed = std::stoul(argv[6]);
    Real3 field{0, 0, 0};
    bool msc = false;
    size_type threads = 1;
    size_type max_steps = 100000;
    std::string rz_field;
    for (int i = 7; i < argc; ++i)
    {
        std::string a = argv[i];
        if (a == "--field")
        {
            field = {std::strtod(argv[i + 1], nullptr),
                     std::strtod(argv[i + 2], nullptr),
                     std::strtod(argv[i + 3], nullptr)};
            i += 3;
        }
        else if (a == "--msc")
            msc = true;
        else if (a == "--threads")
            threads = std::stoul(argv[++i]);
        else if (a == "--max-steps")
            max_steps = std::stoul(argv[++i]);
        else if (a == "--rz-field")
            rz_field = argv[++i];
    }
    KvFile kv(phys_path);
    ImportData imported = load_import(kv, msc);
    Problem prob = build_problem(imported,
                                 geo_name,
                                 seed,
                                 field,
                                 msc,
                                 TrackOrder::none,
                                 false,
                                 rz_field,
                                 threads);
    auto primaries = load_primaries(prim_path, *prob.core->particle());
    std::map<size_type, std::vector<Primary>> events;
    for (auto const& p : primaries)
        events[p.event_id.unchecked_get()].push_back(p);
    std::vector<std::vector<Primary>> ev_list;
    for (auto& kv_ev : events)
    {
        for (auto& p : kv_ev.second)
            p.event_id = EventId{0};
        ev_list.push_back(std::move(kv_ev.second));
    }
    std::vector<unsigned long long> steps(threads, 0);
    std::vector<size_type> done(threads, 0), capped(threads, 0);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (size_type t = 0; t < threads; ++t)
    {
        pool.emplace_back([&, t] {
            StepperInput sinp;
            sinp.params = prob.core;
            sinp.stream_id = StreamId{t};
            sinp.num_track_slots = num_slots;
            Stepper<MemSpace::host> step(std::move(sinp));
            for (std::size_t e = t; e < ev_list.size(); e += threads)
            {
                StepperResult c = step(make_span(ev_list[e]));
                steps[t] += c.active;
                size_type iter = 1;
                while (c && iter < max_steps)
                {
                    c = step();
                    steps[t] += c.active;
                    ++iter;
                }
                if (c)
                {
                    // celer-sim ends a run at its step limit by killing
                    // the tracks still in flight
                    step.kill_active();
                    while (c)
                        c = step();
                    ++capped[t];
                }
                ++done[t];
            }
        });
    }
    for (auto& th : pool)
        th.join();
    auto t1 = std::chrono::steady_clock::now();
    unsigned long long total = 0;
    size_type nev = 0, ncap = 0;
    for (size_type t = 0; t < threads; ++t)
    {
        total += steps[t];
        nev += done[t];
        ncap += capped[t];
    }
    double sec = std::chrono::duration<double>(t1 - t0).count();
    std::printf("bench threads %u events %u track_steps %llu seconds %.6f capped %u\n",
                static_cast<unsigned>(threads),
                nev,
                total,
                sec,
                ncap);
    return 0;
}

int dump_geo(int argc, char** argv)
{
    if (argc < 4)
        return 2;
    GeoSpec spec = build_geometry(argv[3]);
    auto const& host = spec.geo->host_ref();
    std::printf("volumes %zu\n", static_cast<std::size_t>(spec.geo->num_volumes()));
    for (auto vid : range(VolumeId{spec.geo->num_volumes()}))
    {
        std::printf("volume %u %s\n",
                    vid.unchecked_get(),
                    spec.geo->volumes().at(vid).name.c_str());
    }
    std::printf("surfaces %zu\n", static_cast<std::size_t>(host.surface_types.size()));
    for (auto i : range(host.surface_types.size()))
    {
        std::printf("surface %zu type %d\n",
                    static_cast<std::size_t>(i),
                    static_cast<int>(host.surface_types[ItemId<SurfaceType>(i)]));
    }
    {
        auto const& unit = host.simple_units[SimpleUnitId{0}];
        std::printf("background %u\n", unit.background.unchecked_get());
        for (auto i : range(unit.volumes.size()))
        {
            auto const& vr
                = host.volume_records[unit.volumes[LocalVolumeId(i)]];
            std::printf("volrec %zu flags %d maxisect %d faces",
                        static_cast<std::size_t>(i),
                        static_cast<int>(vr.flags),
                        static_cast<int>(vr.max_intersections));
            for (auto f : vr.faces)
            {
                std::printf(" %u", host.local_surface_ids[f].unchecked_get());
            }
            std::printf(" logic");
            for (auto l : vr.logic)
            {
                std::printf(" %d", static_cast<int>(host.logic_ints[l]));
            }
            std::printf("\n");
        }
        for (auto s : range(unit.surfaces.types.size()))
        {
            auto const& surfs = unit.surfaces;
            auto t = host.surface_types[surfs.types[s]];
            auto off = host.real_ids[surfs.data_offsets[s]];
            std::printf("surf %zu type %d data %.17g %.17g\n",
                        static_cast<std::size_t>(s),
                        static_cast<int>(t),
                        host.reals[off],
                        host.reals[off + 1]);
        }
        for (auto s : range(unit.connectivity.size()))
        {
            auto const& conn
                = host.connectivity_records[unit.connectivity[s]];
            std::printf("conn %zu", static_cast<std::size_t>(s));
            for (auto v : conn.neighbors)
            {
                std::printf(" %u", host.local_volume_ids[v].unchecked_get());
            }
            std::printf("\n");
        }
    }
    std::printf("reals %zu\n", static_cast<std::size_t>(host.reals.size()));
    for (auto i : range(host.reals.size()))
    {
        std::printf("real %zu %.17g\n",
                    static_cast<std::size_t>(i),
                    host.reals[ItemId<real_type>(i)]);
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 2)
    {
        std::cerr << "usage: ref_harness {run|geo} ...\n";
        return 2;
    }
    std::string mode = argv[1];
    try
    {
        if (mode == "run")
            return run(argc, argv);
        if (mode == "geo")
            return dump_geo(argc, argv);
        if (mode == "bench")
            return bench(argc, argv);
        if (mode == "interact")
            return interact(argc, argv);
        if (mode == "along")
            return along(argc, argv);
    }
    catch (std::exception const& e)
    {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    std::cerr << "unknown mode " << mode << "\n";
    return 2;
}
