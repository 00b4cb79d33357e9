// Construction of the flattened parameter tables.
//
// The derived quantities are computed with the same expressions as the
// reference's parameter classes so that device lookups reproduce the
// reference's values:
//   elements/materials  src/celeritas/mat/MaterialParams.cc (append_*_def),
//                       src/celeritas/mat/detail/Utils.cc
//   fluctuations        src/celeritas/em/params/FluctuationParams.cc
//   physics tables      src/celeritas/phys/PhysicsParams.cc:280-636,
//                       src/celeritas/grid/ValueGridBuilder.cc
//   model data          src/celeritas/em/model/SeltzerBergerModel.cc (argmax),
//                       src/celeritas/em/model/detail/LivermoreXsInserter.hh
//   geometry            the ORANGE unit that orangeinp builds for the same
//                       boxes (surface dedup, face order, connectivity)
#include "HostParams.hh"

#include <algorithm>
#include <sstream>
#include <tuple>
#include <array>
#include <cmath>
#include <fstream>
#include <map>
#include <stdexcept>

#include "KvFile.hh"
#include "../gbx/Random.hh"

namespace gbx
{
namespace
{
//---------------------------------------------------------------------------//
// Element data tables
//---------------------------------------------------------------------------//
//! Coulomb correction f(Z) = a^2 sum_n 1/(n (n^2 + a^2)), a = alpha Z,
//! evaluated with the series in zeta(2k+1) - 1 (Davies-Bethe-Maximon).
double calc_coulomb_correction(int z)
{
    // zeta(2k+1) - 1 for k = 1..16
    static double const zeta[] = {2.0205690315959429e-01,
                                  3.6927755143369927e-02,
                                  8.3492773819228271e-03,
                                  2.0083928260822143e-03,
                                  4.9418860411946453e-04,
                                  1.2271334757848915e-04,
                                  3.0588236307020493e-05,
                                  7.6371976378997626e-06,
                                  1.9082127165539390e-06,
                                  4.7693298678780645e-07,
                                  1.1921992596531106e-07,
                                  2.9803503514652279e-08,
                                  7.4507117898354301e-09,
                                  1.8626597235130491e-09,
                                  4.6566290650337837e-10,
                                  1.1641550172700519e-10};
    double const alphazsq = ipow<2>(constants::alpha_fine_structure * z);
    double fz = 1 / (1 + alphazsq);
    double azpow = 1;
    for (double zeta_i : zeta)
    {
        fz += azpow * zeta_i;
        azpow *= -alphazsq;
    }
    return alphazsq * fz;
}

//! Mass radiation coefficient 1/(X0 rho) from Tsai's formula
double calc_mass_rad_coeff(ElementRecord const& el)
{
    double const z_real = el.z;
    double lrad, lrad_prime;
    switch (el.z)
    {
        case 1:
            lrad = 5.31;
            lrad_prime = 6.144;
            break;
        case 2:
            lrad = 4.79;
            lrad_prime = 5.621;
            break;
        case 3:
            lrad = 4.74;
            lrad_prime = 5.805;
            break;
        case 4:
            lrad = 4.71;
            lrad_prime = 5.924;
            break;
        default:
            lrad = gbx::libm::log(184.15 * std::pow(z_real, double(-1) / 3));
            lrad_prime = gbx::libm::log(1194.0 * std::pow(z_real, double(-2) / 3));
    }
    constexpr double inv_x0_factor = 4 * constants::alpha_fine_structure
                                     * ipow<2>(constants::r_electron);
    return inv_x0_factor / (el.atomic_mass * constants::atomic_mass)
           * (ipow<2>(z_real) * (lrad - el.coulomb_correction)
              + z_real * lrad_prime);
}

//! Mean excitation energies [eV] by Z (ICRU Report 37 elemental values)
double mean_excitation_energy(int z)
{
    static double const table[] = {
        19.2,  41.8,  40.0,  63.7,  76.0,  81.0,  82.0,  95.0,  115.0, 137.0,
        149.0, 156.0, 166.0, 173.0, 173.0, 180.0, 174.0, 188.0, 190.0, 191.0,
        216.0, 233.0, 245.0, 257.0, 272.0, 286.0, 297.0, 311.0, 322.0, 330.0,
        334.0, 350.0, 347.0, 348.0, 343.0, 352.0, 363.0, 366.0, 379.0, 393.0,
        417.0, 424.0, 428.0, 441.0, 449.0, 470.0, 470.0, 469.0, 488.0, 488.0,
        487.0, 485.0, 491.0, 482.0, 488.0, 491.0, 501.0, 523.0, 535.0, 546.0,
        560.0, 574.0, 580.0, 591.0, 614.0, 628.0, 650.0, 658.0, 674.0, 684.0,
        694.0, 705.0, 718.0, 727.0, 736.0, 746.0, 757.0, 790.0, 790.0, 800.0,
        810.0, 823.0, 823.0, 830.0, 825.0, 794.0, 827.0, 826.0, 841.0, 847.0,
        878.0, 890.0, 902.0, 921.0, 934.0, 939.0, 952.0, 966.0};
    if (z < 1 || z > 98)
        throw std::runtime_error("no mean excitation energy for Z");
    return 1e-6 * table[z - 1];
}

bool soft_equal(double a, double b, double rel = 1e-12, double abs = 1e-14)
{
    double diff = std::fabs(a - b);
    if (diff < abs)
        return true;
    return diff < rel * std::max(std::fabs(a), std::fabs(b));
}

//---------------------------------------------------------------------------//
// Process/model catalog
//---------------------------------------------------------------------------//
// Process IDs follow the order of the reference's import process class enum
// (e_ioni, e_brems, photoelectric, compton, conversion, annihilation)
enum ProcessId : size_type
{
    proc_e_ioni = 0,
    proc_e_brems,
    proc_photoelectric,
    proc_compton,
    proc_conversion,
    proc_annihilation,
    proc_size
};

// Model IDs in the order the processes build them
enum ModelId : size_type
{
    model_moller_bhabha = 0,
    model_seltzer_berger,
    model_rel_brems,
    model_livermore_pe,
    model_klein_nishina,
    model_bethe_heitler,
    model_eplusgg,
    model_size
};

struct Applic
{
    size_type particle;
    double lower;
    double upper;
};

class Builder
{
  public:
    Builder(KvFile const& kv, GeometrySpec const& geo, ParamsOptions const& opts)
        : kv_(kv), geo_(geo), opts_(opts)
    {
    }

    HostParams build();

  private:
    KvFile const& kv_;
    GeometrySpec const& geo_;
    ParamsOptions const& opts_;
    HostParams hp_;
    //! Registered model index of each model kind (the combined
    //! bremsstrahlung model stands for both bremsstrahlung kinds)
    size_type model_index_[model_size];

    size_type add_reals(std::vector<double> const& v)
    {
        size_type off = hp_.reals.size();
        hp_.reals.insert(hp_.reals.end(), v.begin(), v.end());
        return off;
    }
    size_type add_ints(std::vector<size_type> const& v)
    {
        size_type off = hp_.ints.size();
        hp_.ints.insert(hp_.ints.end(), v.begin(), v.end());
        return off;
    }
    //! Insert a log-uniform grid from an imported (x, y) vector
    size_type add_log_grid(std::vector<double> const& x,
                           std::vector<double> const& y);
    GenericGrid add_generic(std::vector<double> const& x,
                            std::vector<double> const& y)
    {
        GenericGrid g;
        g.x = this->add_reals(x);
        g.y = this->add_reals(y);
        g.size = static_cast<size_type>(x.size());
        return g;
    }

    void build_actions();
    void build_msc_field();
    void build_particles();
    void read_rzmap(std::string const& path);
    void build_materials();
    void build_physics();
    void build_models();
    void build_element_tables();
    void build_geometry();
};

size_type Builder::add_log_grid(std::vector<double> const& x,
                                std::vector<double> const& y)
{
    if (x.size() < 2 || x.size() != y.size() || !(x.front() > 0))
        throw std::runtime_error("invalid log grid");
    XsGrid g;
    g.log_front = gbx::libm::log(x.front());
    g.log_back = gbx::libm::log(x.back());
    g.size = static_cast<size_type>(x.size());
    g.log_delta = (g.log_back - g.log_front) / (g.size - 1);
    g.prime_index = invalid_id;
    g.value = this->add_reals(y);
    std::vector<double> energies(g.size + 1);
    for (size_type i = 0; i < g.size; ++i)
    {
        energies[i] = gbx::libm::exp(g.log_front + g.log_delta * i);
    }
    energies[g.size] = gbx::libm::exp(g.log_back);
    g.energy = this->add_reals(energies);
    size_type id = static_cast<size_type>(hp_.grids.size());
    hp_.grids.push_back(g);
    return id;
}

//---------------------------------------------------------------------------//
void Builder::build_actions()
{
    // Registration order of CoreParams/PhysicsParams/Runner (action IDs).
    // The bremsstrahlung process builds either the Seltzer-Berger and the
    // relativistic models or, with brem_combined, one combined model
    // (BremsstrahlungProcess.cc:70-95), which shifts every later ID
    bool const combined = opts_.brem_combined;
    hp_.action_labels = {"pre-step",
                         "msc-range",
                         "eloss-range",
                         "physics-discrete-select",
                         "physics-integral-rejected",
                         "ioni-moller-bhabha"};
    if (combined)
    {
        hp_.action_labels.push_back("brems-combined");
    }
    else
    {
        hp_.action_labels.push_back("brems-sb");
        hp_.action_labels.push_back("brems-rel");
    }
    for (char const* label : {"photoel-livermore",
                              "scat-klein-nishina",
                              "conv-bethe-heitler",
                              "annihil-2-gamma",
                              "physics-failure",
                              "along-step-general-linear",
                              "extend-from-primaries",
                              "initialize-tracks",
                              "along-step-neutral",
                              "geo-propagation-limit",
                              "geo-boundary",
                              "tracking-cut",
                              "extend-from-secondaries"})
    {
        hp_.action_labels.push_back(label);
    }
    ParamsData& s = hp_.scalars;
    // Optional track-sorting actions (CoreParams.cc:258-283): the step-limit
    // sort is registered before the along-step sort
    s.track_order = opts_.track_order;
    s.action_sort_along = s.action_sort_post = s.action_sort_start = invalid_id;
    switch (opts_.track_order)
    {
        case track_order_none:
        case track_order_init_charge:
        case track_order_reindex_shuffle:
            // No sort action: the charge partition is part of the track
            // initialization, the shuffle is done once with the state
            // (CoreParams.cc:264-269, CoreTrackData.cc:47-56)
            break;
        case track_order_reindex_status:
            s.action_sort_start = hp_.action_labels.size();
            hp_.action_labels.push_back("sort-tracks-status");
            break;
        case track_order_reindex_particle_type:
            s.action_sort_start = hp_.action_labels.size();
            hp_.action_labels.push_back("sort-tracks-start");
            break;
        case track_order_reindex_along_step_action:
            s.action_sort_along = hp_.action_labels.size();
            hp_.action_labels.push_back("sort-tracks-along-step");
            break;
        case track_order_reindex_step_limit_action:
            s.action_sort_post = hp_.action_labels.size();
            hp_.action_labels.push_back("sort-tracks-post-step");
            break;
        case track_order_reindex_both_action:
            s.action_sort_post = hp_.action_labels.size();
            hp_.action_labels.push_back("sort-tracks-post-step");
            s.action_sort_along = hp_.action_labels.size();
            hp_.action_labels.push_back("sort-tracks-along-step");
            break;
        default:
            throw std::runtime_error("track order " + std::to_string(opts_.track_order)
                                     + " is not a TrackOrder (0-7)");
    }
    hp_.action_labels.push_back("step-gather-pre");
    hp_.action_labels.push_back("step-gather-post");
    s.num_actions = hp_.action_labels.size();
    auto id = [this](char const* label) {
        auto const& v = hp_.action_labels;
        return static_cast<size_type>(std::find(v.begin(), v.end(), label) - v.begin());
    };
    s.action_pre_step = id("pre-step");
    s.action_msc_range = id("msc-range");
    s.action_range = id("eloss-range");
    s.action_discrete = id("physics-discrete-select");
    s.action_integral_rejection = id("physics-integral-rejected");
    // Registered models: IDs in registration order, the model actions
    // following each other from model_to_action
    s.model_to_action = id("ioni-moller-bhabha");
    size_type next = 0;
    model_index_[model_moller_bhabha] = next++;
    model_index_[model_seltzer_berger] = next++;
    model_index_[model_rel_brems] = combined ? model_index_[model_seltzer_berger] : next++;
    for (ModelId m : {model_livermore_pe, model_klein_nishina, model_bethe_heitler,
                      model_eplusgg})
    {
        model_index_[m] = next++;
    }
    s.num_models = next;
    s.action_moller_bhabha = id("ioni-moller-bhabha");
    s.action_seltzer_berger = combined ? invalid_id : id("brems-sb");
    s.action_rel_brems = combined ? invalid_id : id("brems-rel");
    s.action_combined_brems = combined ? id("brems-combined") : invalid_id;
    s.action_livermore_pe = id("photoel-livermore");
    s.action_klein_nishina = id("scat-klein-nishina");
    s.action_bethe_heitler = id("conv-bethe-heitler");
    s.action_eplusgg = id("annihil-2-gamma");
    s.action_failure = id("physics-failure");
    s.action_along_step = id("along-step-general-linear");
    s.action_along_step_neutral = id("along-step-neutral");
    s.action_propagation_limit = id("geo-propagation-limit");
    s.action_boundary = id("geo-boundary");
    s.action_tracking_cut = id("tracking-cut");
}

void Builder::build_particles()
{
    long npar = kv_.i("particles");
    ParamsData& s = hp_.scalars;
    s.electron_id = s.positron_id = s.gamma_id = invalid_id;
    for (long i = 0; i < npar; ++i)
    {
        auto const& v = kv_.get("particle." + std::to_string(i));
        ParticleRecord pr;
        pr.pdg = std::stoi(v[1]);
        pr.mass = std::strtod(v[2].c_str(), nullptr);
        pr.charge = std::strtod(v[3].c_str(), nullptr);
        pr.is_antiparticle = pr.pdg < 0;
        if (pr.pdg == 11)
            s.electron_id = i;
        else if (pr.pdg == -11)
            s.positron_id = i;
        else if (pr.pdg == 22)
            s.gamma_id = i;
        hp_.particles.push_back(pr);
    }
    if (s.electron_id != 0 || s.positron_id != 1 || s.gamma_id != 2)
        throw std::runtime_error("expected particles e-, e+, gamma in order");
    s.num_particles = static_cast<size_type>(npar);
    // The reference's particle order: increasing mass, then |PDG|, then
    // particles before antiparticles
    std::vector<size_type> order(hp_.particles.size());
    for (size_type i = 0; i < order.size(); ++i)
        order[i] = i;
    auto key = [this](size_type i) {
        auto const& pr = hp_.particles[i];
        return std::make_tuple(double(pr.mass), std::abs(pr.pdg), pr.pdg < 0);
    };
    std::sort(order.begin(), order.end(), [&key](size_type a, size_type b) {
        return key(a) < key(b);
    });
    for (size_type r = 0; r < order.size(); ++r)
        hp_.particles[order[r]].ref_id = r;
}

void Builder::build_materials()
{
    long nel = kv_.i("elements");
    for (long i = 0; i < nel; ++i)
    {
        auto p = "element." + std::to_string(i);
        ElementRecord el;
        el.z = static_cast<int>(kv_.i(p + ".z"));
        el.atomic_mass = kv_.d(p + ".a");
        double const z_real = el.z;
        el.cbrt_z = gbx::libm::cbrt(z_real);
        el.cbrt_zzp = gbx::libm::cbrt(z_real * (z_real + 1));
        el.log_z = gbx::libm::log(z_real);
        el.coulomb_correction = calc_coulomb_correction(el.z);
        el.mass_radiation_coeff = calc_mass_rad_coeff(el);
        hp_.elements.push_back(el);
    }

    long nmat = kv_.i("materials");
    double const electron_mass = hp_.particles[hp_.scalars.electron_id].mass;
    for (long i = 0; i < nmat; ++i)
    {
        auto p = "material." + std::to_string(i);
        hp_.material_labels.push_back(kv_.s(p + ".name"));
        MaterialRecord m{};
        m.number_density = kv_.d(p + ".number_density");
        auto els = kv_.dbl(p + ".elements");
        auto fr = kv_.dbl(p + ".fractions");
        if (els.size() > max_elements)
            throw std::runtime_error("too many elements in material");
        // Sort components by element ID; renormalize if they don't sum to 1
        std::vector<std::pair<size_type, double>> comps;
        double norm = 0;
        for (std::size_t j = 0; j < els.size(); ++j)
        {
            comps.push_back({static_cast<size_type>(els[j]), fr[j]});
            norm += fr[j];
        }
        if (!comps.empty() && !soft_equal(norm, 1.0))
        {
            norm = 1 / norm;
            for (auto& c : comps)
                c.second *= norm;
        }
        std::sort(comps.begin(), comps.end(), [](auto const& a, auto const& b) {
            return a.first < b.first;
        });
        m.num_elements = static_cast<size_type>(comps.size());
        double avg_amu_mass = 0;
        double avg_z = 0;
        double rad_coeff = 0;
        double log_mean_exc_energy = 0;
        for (std::size_t j = 0; j < comps.size(); ++j)
        {
            m.element[j] = comps[j].first;
            m.fraction[j] = comps[j].second;
            ElementRecord const& el = hp_.elements[comps[j].first];
            double frac_z = comps[j].second * el.z;
            avg_amu_mass += comps[j].second * el.atomic_mass;
            avg_z += frac_z;
            rad_coeff += comps[j].second * el.mass_radiation_coeff;
            log_mean_exc_energy
                += frac_z * gbx::libm::log(mean_excitation_energy(el.z));
        }
        m.zeff = avg_z;
        m.density = m.number_density * avg_amu_mass * constants::atomic_mass;
        m.electron_density = m.number_density * avg_z;
        m.rad_length = 1 / (rad_coeff * m.density);
        log_mean_exc_energy = avg_z > 0 ? log_mean_exc_energy / avg_z
                                        : -INFINITY;
        m.log_mean_exc_energy = log_mean_exc_energy;
        m.mean_exc_energy = gbx::libm::exp(log_mean_exc_energy);
        hp_.materials.push_back(m);

        // Urban fluctuation parameters
        UrbanFluctRecord f;
        double const avg_zf = m.electron_density / m.number_density;
        f.oscillator_strength[1] = avg_zf > 2 ? 2 / avg_zf : 0;
        f.oscillator_strength[0] = 1 - f.oscillator_strength[1];
        f.binding_energy[1] = 1e-5 * ipow<2>(avg_zf);
        f.binding_energy[0]
            = std::pow(m.mean_exc_energy
                           / std::pow(f.binding_energy[1], f.oscillator_strength[1]),
                       1 / f.oscillator_strength[0]);
        f.log_binding_energy[1] = gbx::libm::log(f.binding_energy[1]);
        f.log_binding_energy[0] = gbx::libm::log(f.binding_energy[0]);
        hp_.fluct.push_back(f);

        // Production cutoffs per particle
        for (auto const& par : hp_.particles)
        {
            auto c = kv_.dbl(p + ".cut." + std::to_string(par.pdg));
            hp_.cutoffs.push_back(c.at(0));
        }
    }
    (void)electron_mass;
    hp_.scalars.num_materials = static_cast<size_type>(nmat);
}

void Builder::build_physics()
{
    ParamsData& s = hp_.scalars;
    if (!opts_.field_options.valid())
        throw std::runtime_error("invalid field driver options");
    s.field_options = opts_.field_options;
    // PhysicsParamsOptions defaults and imported EM parameters
    s.min_range = 1 * constants::millimeter;
    s.max_step_over_range = 0.2;
    s.min_eprime_over_e = 0.8;
    s.linear_loss_limit = kv_.d("em.linear_loss_limit");
    s.lowest_electron_energy = kv_.d("em.lowest_electron_energy");
    s.secondary_stack_factor = opts_.secondary_stack_factor;
    s.enable_fluct = kv_.i("em.energy_loss_fluct") != 0;
    s.enable_lpm = kv_.i("em.lpm") != 0;
    bool const integral = kv_.i("em.integral_approach") != 0;
    s.photoelectric_process = proc_photoelectric;
    s.annihilation_process = proc_annihilation;
    s.photoelectric_table_thresh = 0.2;
    s.livermore_model = model_index_[model_livermore_pe];
    s.eplusgg_model = model_index_[model_eplusgg];

    double const electron_mass = hp_.particles[s.electron_id].mass;
    double const max_e = INFINITY;
    size_type const e = s.electron_id, ep = s.positron_id, g = s.gamma_id;

    // Model applicability (hardcoded in the reference's model classes)
    struct ModelDef
    {
        ModelId model;
        ProcessId process;
        std::vector<Applic> applic;
    };
    double const sb_upper = 1e3;  // seltzer_berger_upper_limit: 1 GeV
    double const high_limit = 1e8;  // 100 TeV
    std::vector<ModelDef> models = {
        {model_moller_bhabha, proc_e_ioni, {{e, 0, 100e6}, {ep, 0, 100e6}}}};
    if (opts_.brem_combined)
    {
        // CombinedBremModel::applicability (CombinedBremModel.cc:67-79): one
        // model over the whole range, which picks Seltzer-Berger or the
        // relativistic sampler per interaction. It has no per-element cross
        // sections, so every material must hold a single element
        // (PhysicsParams.cc:660-668)
        for (auto const& m : hp_.materials)
        {
            if (m.num_elements > 1)
                throw std::runtime_error(
                    "model 'brems-combined' cannot be used with materials composed of "
                    "more than one element");
        }
        models.push_back({model_seltzer_berger,
                          proc_e_brems,
                          {{e, 0, high_limit}, {ep, 0, high_limit}}});
    }
    else
    {
        models.push_back(
            {model_seltzer_berger, proc_e_brems, {{e, 0, sb_upper}, {ep, 0, sb_upper}}});
        models.push_back({model_rel_brems,
                          proc_e_brems,
                          {{e, sb_upper, high_limit}, {ep, sb_upper, high_limit}}});
    }
    models.push_back({model_livermore_pe, proc_photoelectric, {{g, 0, max_e}}});
    models.push_back({model_klein_nishina, proc_compton, {{g, 0, max_e}}});
    models.push_back({model_bethe_heitler, proc_conversion, {{g, 2 * electron_mass, 1e8}}});
    models.push_back({model_eplusgg, proc_annihilation, {{ep, 0, 1e8}}});

    // particle -> process -> [(lower, upper, registered model)]
    std::vector<std::map<size_type, std::vector<std::tuple<double, double, size_type>>>>
        particle_models(hp_.particles.size());
    for (auto const& md : models)
    {
        for (auto const& a : md.applic)
        {
            particle_models[a.particle][md.process].push_back(
                {a.lower, a.upper, model_index_[md.model]});
        }
    }

    // Which processes use the integral approach
    auto uses_integral = [integral](size_type proc) {
        return integral
               && (proc == proc_e_ioni || proc == proc_e_brems
                   || proc == proc_annihilation);
    };
    // Imported table names per process
    auto process_name = [](size_type proc) -> std::string {
        switch (proc)
        {
            case proc_e_ioni: return "e_ioni";
            case proc_e_brems: return "e_brems";
            case proc_photoelectric: return "photoelectric";
            case proc_compton: return "compton";
            case proc_conversion: return "conversion";
            case proc_annihilation: return "annihilation";
        }
        return "";
    };

    size_type const nmat = s.num_materials;
    for (size_type pid = 0; pid < hp_.particles.size(); ++pid)
    {
        ProcessGroup pg{};
        pg.eloss_process = invalid_id;
        for (int v = 0; v < vgt_size; ++v)
            pg.grid_table[v] = invalid_id;
        auto const& procs = particle_models[pid];
        if (procs.size() > max_processes)
            throw std::runtime_error("too many processes");
        pg.num_processes = static_cast<size_type>(procs.size());
        std::vector<std::vector<size_type>> tables(
            vgt_size, std::vector<size_type>(procs.size() * nmat, invalid_id));
        bool any_table[vgt_size] = {false, false, false};
        size_type ppid = 0;
        int pdg = hp_.particles[pid].pdg;
        for (auto const& [proc, mlist_in] : procs)
        {
            auto mlist = mlist_in;
            std::sort(mlist.begin(), mlist.end());
            pg.process[ppid] = proc;
            std::vector<double> egrid{std::get<0>(mlist.front())};
            std::vector<size_type> mids;
            for (auto const& m : mlist)
            {
                if (egrid.back() != std::get<0>(m))
                    throw std::runtime_error("noncontiguous model energies");
                egrid.push_back(std::get<1>(m));
                mids.push_back(std::get<2>(m));
            }
            pg.model_energy[ppid] = this->add_reals(egrid);
            pg.model_ids[ppid] = this->add_ints(mids);
            pg.num_models[ppid] = static_cast<size_type>(mids.size());
            pg.use_integral[ppid] = uses_integral(proc);

            std::vector<double> energy_max_xs(nmat, 0);
            std::string base = "table." + std::to_string(pdg) + "."
                               + process_name(proc) + ".";
            for (size_type mat = 0; mat < nmat; ++mat)
            {
                std::string ms = "." + std::to_string(mat);
                size_type macro = invalid_id;
                if (proc == proc_annihilation)
                {
                    pg.has_at_rest = true;
                }
                else if (kv_.has(base + "lambda" + ms + ".x"))
                {
                    macro = this->add_log_grid(kv_.dbl(base + "lambda" + ms + ".x"),
                                               kv_.dbl(base + "lambda" + ms + ".y"));
                    XsGrid const& xg = hp_.grids[macro];
                    // Discrete interaction at rest if xs(E=0) > 0
                    pg.has_at_rest |= hp_.reals[xg.value] > 0;
                    if (pg.use_integral[ppid])
                    {
                        double xs_max = 0;
                        double e_max = 0;
                        for (size_type i = 0; i < xg.size; ++i)
                        {
                            double xs = hp_.reals[xg.value + i];
                            if (xs > xs_max)
                            {
                                xs_max = xs;
                                e_max = hp_.reals[xg.energy + i];
                            }
                        }
                        energy_max_xs[mat] = e_max;
                    }
                }
                tables[vgt_macro_xs][ppid * nmat + mat] = macro;
                if (macro != invalid_id)
                    any_table[vgt_macro_xs] = true;
                if (kv_.has(base + "dedx" + ms + ".x")
                    && kv_.has(base + "range" + ms + ".x"))
                {
                    tables[vgt_energy_loss][ppid * nmat + mat] = this->add_log_grid(
                        kv_.dbl(base + "dedx" + ms + ".x"),
                        kv_.dbl(base + "dedx" + ms + ".y"));
                    tables[vgt_range][ppid * nmat + mat] = this->add_log_grid(
                        kv_.dbl(base + "range" + ms + ".x"),
                        kv_.dbl(base + "range" + ms + ".y"));
                    any_table[vgt_energy_loss] = any_table[vgt_range] = true;
                    pg.eloss_process = ppid;
                }
            }
            pg.energy_max_xs[ppid]
                = pg.use_integral[ppid] ? this->add_reals(energy_max_xs) : invalid_id;
            ++ppid;
        }
        for (int v = 0; v < vgt_size; ++v)
        {
            if (any_table[v])
                pg.grid_table[v] = this->add_ints(tables[v]);
        }
        hp_.groups.push_back(pg);
    }
}

void Builder::build_models()
{
    // Seltzer-Berger tables per element, with the argmax over reduced energy
    for (auto const& el : hp_.elements)
    {
        std::string z = std::to_string(el.z);
        auto x = kv_.dbl("sb." + z + ".x");
        auto y = kv_.dbl("sb." + z + ".y");
        auto v = kv_.dbl("sb." + z + ".value");
        if (v.size() != x.size() * y.size())
            throw std::runtime_error("bad SB table size");
        SBElementTable t;
        t.x = this->add_reals(x);
        t.nx = static_cast<size_type>(x.size());
        t.y = this->add_reals(y);
        t.ny = static_cast<size_type>(y.size());
        t.values = this->add_reals(v);
        std::vector<size_type> argmax(x.size());
        for (std::size_t i = 0; i < x.size(); ++i)
        {
            auto first = v.begin() + i * y.size();
            argmax[i] = static_cast<size_type>(
                std::max_element(first, first + y.size()) - first);
        }
        t.argmax = this->add_ints(argmax);
        hp_.sb_tables.push_back(t);
    }

    // Relativistic bremsstrahlung element factors (form factors of Tsai for
    // Z < 5, Thomas-Fermi radiation logarithms above)
    {
        double const electron_mass = hp_.particles[hp_.scalars.electron_id].mass;
        static double const form_factor[4][2] = {
            {5.3104, 5.9173}, {4.7935, 5.6125}, {4.7402, 5.5377}, {4.7112, 5.4728}};
        for (auto const& el : hp_.elements)
        {
            int const z = std::min(el.z, 120);
            double ff_el, ff_inel;
            if (z < 5)
            {
                ff_el = form_factor[z - 1][0];
                ff_inel = form_factor[z - 1][1];
            }
            else
            {
                ff_el = double(gbx::libm::log(184.15)) - el.log_z / 3;
                ff_inel = double(gbx::libm::log(1194.0)) - 2 * el.log_z / 3;
            }
            double const fc = el.coulomb_correction;
            double const invz = double(1) / z;
            double const z13 = el.cbrt_z;
            double const z23 = ipow<2>(z13);
            RelBremElementRecord r;
            r.fz = el.log_z / 3 + fc;
            r.factor1 = (ff_el - fc) + ff_inel * invz;
            r.factor2 = (1 + invz) / 12;
            r.gamma_factor = 100 * electron_mass / z13;
            r.epsilon_factor = 100 * electron_mass / z23;
            hp_.rb_elements.push_back(r);
        }
    }

    // Livermore photoelectric data per element
    for (auto const& el : hp_.elements)
    {
        std::string pz = "livermore." + std::to_string(el.z);
        LivermoreElement le{};
        if (kv_.has(pz + ".xs_lo.x"))
        {
            le.xs_lo = this->add_generic(kv_.dbl(pz + ".xs_lo.x"),
                                         kv_.dbl(pz + ".xs_lo.y"));
        }
        le.xs_hi = this->add_generic(kv_.dbl(pz + ".xs_hi.x"),
                                     kv_.dbl(pz + ".xs_hi.y"));
        auto th = kv_.dbl(pz + ".thresh");
        le.thresh_lo = th[0];
        le.thresh_hi = th[1];
        le.shells = static_cast<size_type>(hp_.lv_shells.size());
        long nsh = kv_.i(pz + ".shells");
        le.num_shells = static_cast<size_type>(nsh);
        for (long s = 0; s < nsh; ++s)
        {
            std::string ps = pz + ".shell." + std::to_string(s);
            LivermoreShell sh{};
            sh.binding_energy = kv_.d(ps + ".binding");
            auto lo = kv_.dbl(ps + ".param_lo");
            auto hi = kv_.dbl(ps + ".param_hi");
            for (int i = 0; i < 6; ++i)
            {
                sh.param[0][i] = lo.at(i);
                sh.param[1][i] = hi.at(i);
            }
            sh.xs = this->add_generic(kv_.dbl(ps + ".energy"), kv_.dbl(ps + ".xs"));
            hp_.lv_shells.push_back(sh);
        }
        hp_.lv_elements.push_back(le);
    }
}

//! R-Z field map (RZMapFieldParams::RZMapFieldParams,
//! src/celeritas/field/RZMapFieldParams.cc): header 'rzmap num_z num_r
//! min_z max_z min_r max_r' [cm], then 'Bz Br' [tesla] per node, [z][r]
void Builder::read_rzmap(std::string const& path)
{
    std::ifstream in(path);
    if (!in)
        throw std::runtime_error("cannot open field map " + path);
    std::string tag;
    unsigned int nz = 0, nr = 0;
    double min_z, max_z, min_r, max_r;
    in >> tag >> nz >> nr >> min_z >> max_z >> min_r >> max_r;
    if (!in || tag != "rzmap")
        throw std::runtime_error("bad field map header in " + path);
    if (nz < 2 || nr < 2 || !(min_r >= 0) || !(max_r > min_r) || !(max_z > min_z))
        throw std::runtime_error("invalid field map grid in " + path);
    hp_.rzmap.resize(std::size_t(nz) * nr);
    for (auto& el : hp_.rzmap)
    {
        double bz, br;
        if (!(in >> bz >> br))
            throw std::runtime_error("truncated field map " + path);
        el.value_z = bz * constants::tesla;
        el.value_r = br * constants::tesla;
    }
    auto grid = [](double lo, double hi, unsigned int n) {
        FieldMapGrid g;
        g.front = lo;
        g.back = hi;
        g.delta = (hi - lo) / (n - 1);
        g.size = n;
        return g;
    };
    hp_.rzmap_desc.z = grid(min_z, max_z, nz);
    hp_.rzmap_desc.r = grid(min_r, max_r, nr);
    hp_.rzmap_desc.values = hp_.rzmap.data();
    hp_.rzmap_f.resize(hp_.rzmap.size());
    for (std::size_t i = 0; i < hp_.rzmap.size(); ++i)
    {
        hp_.rzmap_f[i] = {static_cast<float>(hp_.rzmap[i].value_z),
                          static_cast<float>(hp_.rzmap[i].value_r)};
    }
    hp_.rzmap_desc.values_f = hp_.rzmap_f.data();
}

void Builder::build_msc_field()
{
    ParamsData& s = hp_.scalars;
    // Field (UniformFieldParams: input in tesla, stored in native units)
    s.has_field = false;
    for (int i = 0; i < 3; ++i)
    {
        s.field[i] = opts_.field_tesla[i] * constants::tesla;
        if (s.field[i] != 0)
            s.has_field = true;
    }
    if (s.has_field)
        hp_.action_labels[s.action_along_step] = "along-step-uniform-msc";
    s.has_rzmap = false;
    if (!opts_.rz_field_file.empty())
    {
        if (s.has_field)
            throw std::runtime_error("an R-Z field map excludes a uniform field");
        this->read_rzmap(opts_.rz_field_file);
        s.has_field = s.has_rzmap = true;
        hp_.action_labels[s.action_along_step] = "along-step-rzmap-msc";
    }

    // Looping thresholds (SimParams::from_import with 10 field substeps)
    {
        auto lp = kv_.dbl("trans.looping");
        long const max_substeps = kv_.i("trans.max_substeps");
        size_type const field_substeps = 10;
        size_type const max_subthreshold
            = (static_cast<size_type>(max_substeps) + field_substeps - 1)
              / field_substeps;
        hp_.looping.assign(hp_.particles.size(), LoopingRecord{});
        for (std::size_t j = 0; j + 2 < lp.size() + 0; j += 3)
        {
            int pdg = static_cast<int>(lp[j]);
            for (std::size_t pid = 0; pid < hp_.particles.size(); ++pid)
            {
                if (hp_.particles[pid].pdg != pdg)
                    continue;
                LoopingRecord& r = hp_.looping[pid];
                r.max_subthreshold_steps = max_subthreshold;
                r.max_steps = static_cast<size_type>(lp[j + 1]) * max_subthreshold;
                r.threshold_energy = lp[j + 2];
            }
        }
    }

    // Urban multiple scattering (UrbanMscParams)
    UrbanMscParams& m = s.msc;
    m.enabled = opts_.msc;
    m.lambda_limit = 1 * constants::millimeter;
    m.range_factor = 0.04;
    m.safety_factor = 0.6;
    m.xs_grids = invalid_id;
    if (!opts_.msc)
        return;
    auto poly2 = [](double c0, double c1, double c2, double x) {
        double const c[3] = {c0, c1, c2};
        return poly_eval<2>(c, x);
    };
    std::vector<size_type> grids;
    static double const a_coeff[2] = {0.87, 0.70};
    static double const b_coeff[2] = {2.0 / 3, 1.0 / 2};
    for (size_type mid = 0; mid < hp_.materials.size(); ++mid)
    {
        double const zeff = hp_.materials[mid].zeff;
        UrbanMscMaterialRecord md;
        md.stepmin_coeff[0] = 1e3 * 27.725 / (1 + 0.203 * zeff);
        md.stepmin_coeff[1] = 1e3 * 6.152 / (1 + 0.111 * zeff);
        double const z16 = gbx::libm::exp(1.0 / 6.0 * gbx::libm::log(zeff));
        double fz = poly2(0.990395, -0.168386, 0.093286, z16);
        md.theta_coeff[0] = fz * (1 - 8.7780e-2 / zeff);
        md.theta_coeff[1] = fz * (4.0780e-2 + 1.7315e-4 * zeff);
        double z13 = ipow<2>(z16);
        md.tail_coeff[0] = poly2(2.3785, -4.1981e-1, 6.3100e-2, z13);
        md.tail_coeff[1] = poly2(4.7526e-1, 1.7694, -3.3885e-1, z13);
        md.tail_coeff[2] = poly2(2.3683e-1, -1.8111, 3.2774e-1, z13);
        md.tail_corr = poly2(1.7888e-2, 1.9659e-2, -2.6664e-3, z13);
        hp_.msc_materials.push_back(md);
        for (int pi = 0; pi < 2; ++pi)
        {
            UrbanMscParMatRecord pm;
            pm.scaled_zeff = a_coeff[pi] * gbx::libm::exp(b_coeff[pi] * gbx::libm::log(zeff));
            pm.d_over_r = 9.6280e-1 - 8.4848e-2 * std::sqrt(zeff) + 4.3769e-3 * zeff;
            hp_.msc_par_mat.push_back(pm);
            int pdg = (pi == 0) ? 11 : -11;
            std::string key = "msc." + std::to_string(pdg) + "." + std::to_string(mid);
            grids.push_back(this->add_log_grid(kv_.dbl(key + ".x"), kv_.dbl(key + ".y")));
        }
    }
    m.xs_grids = this->add_ints(grids);
    auto x = kv_.dbl("msc.11.0.x");
    m.low_energy_limit = x.front();
    m.high_energy_limit = x.back();
}

void Builder::build_geometry()
{
    // Surfaces: world box faces, then each volume's surfaces in insertion
    // order, deduplicated against existing surfaces (first inserted wins).
    // Each box face is placed at center +/- half-width, as a translated box;
    // a shell inserts its z planes, outer cylinder, then inner cylinder.
    auto add_surface = [this](int type, double value) -> size_type {
        for (size_type i = 0; i < hp_.surfaces.size(); ++i)
        {
            auto const& sr = hp_.surfaces[i];
            if (sr.type == type
                && std::fabs(sr.value - value)
                       <= 1e-8 * std::max(1.0, std::fabs(value)))
            {
                return i;
            }
        }
        float const radius
            = (type == surf_czc) ? static_cast<float>(std::sqrt(value)) : 0.0f;
        double const radius_d = (type == surf_czc) ? std::sqrt(value) : 0.0;
        hp_.surfaces.push_back({type, radius, value, radius_d});
        return static_cast<size_type>(hp_.surfaces.size() - 1);
    };
    auto box_faces = [&](double const* lo, double const* hi, size_type* faces) {
        for (int ax = 0; ax < 3; ++ax)
        {
            double half = (hi[ax] - lo[ax]) / 2;
            double center = (hi[ax] + lo[ax]) / 2;
            faces[2 * ax] = add_surface(ax, -half + center);
            faces[2 * ax + 1] = add_surface(ax, half + center);
        }
    };
    // Faces sorted by surface ID with their inside senses
    auto set_faces = [](VolumeRecord* vr,
                        std::vector<std::pair<size_type, std::int8_t>> fs) {
        std::sort(fs.begin(), fs.end());
        vr->num_faces = static_cast<size_type>(fs.size());
        for (size_type f = 0; f < fs.size(); ++f)
        {
            vr->faces[f] = fs[f].first;
            vr->inside_sense[f] = fs[f].second;
        }
    };

    GeoParams& g = hp_.scalars.geo;
    size_type world[6];
    box_faces(geo_.world_lo, geo_.world_hi, world);
    for (int f = 0; f < 6; ++f)
    {
        g.world_faces[f] = world[f];
        g.world_sense[f] = (f % 2 == 0) ? 1 : -1;
    }
    if (!geo_.boxes.empty() && !geo_.shells.empty())
        throw std::runtime_error("a geometry holds either boxes or shells");

    // Volumes: exterior (0), boxes or shells (1..n), background (n+1)
    size_type const nvol
        = static_cast<size_type>(geo_.boxes.size() + geo_.shells.size());
    hp_.volumes.resize(nvol + 2);
    hp_.volume_labels.push_back("[EXTERIOR]");
    hp_.volume_material.push_back(invalid_id);
    std::vector<std::string> labels;
    for (size_type b = 0; b < geo_.boxes.size(); ++b)
    {
        BoxSpec const& spec = geo_.boxes[b];
        size_type faces[6];
        box_faces(spec.lo, spec.hi, faces);
        // Lower planes need pos >= plane
        std::vector<std::pair<size_type, std::int8_t>> fs;
        for (int f = 0; f < 6; ++f)
            fs.push_back({faces[f], static_cast<std::int8_t>(f % 2 == 0 ? 1 : -1)});
        VolumeRecord& vr = hp_.volumes[b + 1];
        set_faces(&vr, fs);
        vr.material = spec.material;
        labels.push_back(spec.label);
        hp_.volume_material.push_back(spec.material);
    }
    for (size_type k = 0; k < geo_.shells.size(); ++k)
    {
        ShellSpec const& spec = geo_.shells[k];
        if (!(0 < spec.r_in && spec.r_in < spec.r_out && spec.z_lo < spec.z_hi))
            throw std::runtime_error("invalid shell '" + spec.label + "'");
        size_type zlo = add_surface(surf_pz, spec.z_lo);
        size_type zhi = add_surface(surf_pz, spec.z_hi);
        size_type cout = add_surface(surf_czc, spec.r_out * spec.r_out);
        size_type cin = add_surface(surf_czc, spec.r_in * spec.r_in);
        VolumeRecord& vr = hp_.volumes[k + 1];
        set_faces(&vr, {{zlo, 1}, {zhi, -1}, {cout, -1}, {cin, 1}});
        vr.material = spec.material;
        labels.push_back(spec.label);
        hp_.volume_material.push_back(spec.material);
    }
    hp_.volume_labels.insert(hp_.volume_labels.end(), labels.begin(), labels.end());
    hp_.volume_labels.push_back("world");
    hp_.volume_material.push_back(geo_.background_material);

    if (geo_.shells.empty())
    {
        // Box lookup along z requires the lower z face in slot 4 and boxes
        // sorted by it
        g.locate = locate_stack_z;
        for (size_type b = 1; b <= nvol; ++b)
        {
            VolumeRecord const& vr = hp_.volumes[b];
            auto const& sr = hp_.surfaces[vr.faces[4]];
            if (sr.type != surf_pz || vr.inside_sense[4] != 1)
                throw std::runtime_error("boxes must be layered along z");
            if (b > 1
                && !(hp_.surfaces[hp_.volumes[b - 1].faces[4]].value < sr.value))
                throw std::runtime_error("boxes must be sorted along z");
        }
    }
    else
    {
        g.locate = locate_scan;
    }

    // Connectivity: volumes owning each surface
    size_type const nsurf = static_cast<size_type>(hp_.surfaces.size());
    std::vector<std::vector<size_type>> conn(nsurf);
    for (int f = 0; f < 6; ++f)
        conn[world[f]].push_back(0);
    for (size_type b = 1; b <= nvol; ++b)
        for (size_type f = 0; f < hp_.volumes[b].num_faces; ++f)
            conn[hp_.volumes[b].faces[f]].push_back(b);
    hp_.neighbor_offset.push_back(0);
    for (auto const& c : conn)
    {
        hp_.neighbors.insert(hp_.neighbors.end(), c.begin(), c.end());
        hp_.neighbor_offset.push_back(static_cast<size_type>(hp_.neighbors.size()));
    }

    // Surfaces by kind, sorted by value (ties by ID), for the ordered
    // searches of the implicit background
    {
        std::vector<size_type> order(nsurf);
        for (size_type i = 0; i < nsurf; ++i)
            order[i] = i;
        auto const& sf = hp_.surfaces;
        std::sort(order.begin(), order.end(), [&sf](size_type a, size_type b) {
            if (sf[a].type != sf[b].type)
                return sf[a].type < sf[b].type;
            if (sf[a].value != sf[b].value)
                return sf[a].value < sf[b].value;
            return a < b;
        });
        hp_.sorted_surfaces = order;
        hp_.sorted_key.resize(nsurf);
        for (int k = 0; k < 5; ++k)
            g.sorted_offset[k] = 0;
        for (size_type i = 0; i < nsurf; ++i)
        {
            SurfaceRecord const& sr = sf[order[i]];
            if (sr.type < surf_px || sr.type > surf_czc)
                throw std::runtime_error("unknown surface type");
            hp_.sorted_key[i] = (sr.type == surf_czc) ? sr.radius
                                                      : static_cast<float>(sr.value);
            ++g.sorted_offset[sr.type + 1];
        }
        for (int k = 0; k < 4; ++k)
            g.sorted_offset[k + 1] += g.sorted_offset[k];
    }

    // Detectors: every volume, in order
    hp_.volume_detector.assign(nvol + 2, invalid_id);
    for (size_type b = 1; b <= nvol; ++b)
    {
        hp_.volume_detector[b] = b - 1;
        hp_.detector_labels.push_back(labels[b - 1]);
    }

    g.num_surfaces = nsurf;
    g.num_volumes = nvol + 2;
    g.exterior = 0;
    g.background = nvol + 1;
    g.tol_rel = 1.5e-8;
    g.tol_abs = 1.5e-8;
    hp_.scalars.num_detectors = nvol;
}

void Builder::build_element_tables()
{
    // For each model with imported per-element micro cross sections and
    // each material of more than one element: the element-fraction-weighted
    // cumulative cross section, normalized to 1 in each energy bin, one grid
    // per element component (PhysicsParams::build_model_xs,
    // src/celeritas/phys/PhysicsParams.cc:638-768)
    size_type const nmat = static_cast<size_type>(hp_.materials.size());
    size_type const npar = static_cast<size_type>(hp_.particles.size());
    std::vector<size_type> index(std::size_t(hp_.scalars.num_models) * npar * nmat,
                                 invalid_id);
    auto build = [&](ModelId kind, size_type particle, std::string const& prefix) {
        size_type const model = model_index_[kind];
        for (size_type mi = 0; mi < nmat; ++mi)
        {
            MaterialRecord const& m = hp_.materials[mi];
            std::string p = prefix + "." + std::to_string(mi);
            if (m.num_elements <= 1 || !kv_.has(p + ".energy"))
                continue;
            auto energy = kv_.dbl(p + ".energy");
            // Micro cross sections are listed in the input's element order
            auto file_els = kv_.dbl("material." + std::to_string(mi) + ".elements");
            std::vector<std::vector<double>> xs(m.num_elements);
            for (size_type j = 0; j < m.num_elements; ++j)
            {
                std::size_t k = 0;
                while (k < file_els.size()
                       && static_cast<size_type>(file_els[k]) != m.element[j])
                    ++k;
                if (k == file_els.size())
                    throw std::runtime_error("element missing from micro xs");
                xs[j] = kv_.dbl(p + ".micro." + std::to_string(k));
                if (xs[j].size() != energy.size())
                    throw std::runtime_error("bad micro xs size");
            }
            for (std::size_t bin = 0; bin < energy.size(); ++bin)
            {
                double cum_xs = 0;
                for (size_type j = 0; j < m.num_elements; ++j)
                {
                    cum_xs += xs[j][bin] * m.fraction[j];
                    xs[j][bin] = cum_xs;
                }
                if (cum_xs > 0)
                {
                    for (size_type j = 0; j < m.num_elements; ++j)
                        xs[j][bin] /= cum_xs;
                }
            }
            std::vector<size_type> grid_ids(m.num_elements);
            for (size_type j = 0; j < m.num_elements; ++j)
                grid_ids[j] = this->add_log_grid(energy, xs[j]);
            index[(std::size_t(model) * npar + particle) * nmat + mi]
                = this->add_ints(grid_ids);
        }
    };
    ParamsData const& s = hp_.scalars;
    build(model_bethe_heitler, s.gamma_id, "model.22.conversion.bethe_heitler");
    for (size_type pid : {s.electron_id, s.positron_id})
    {
        std::string pdg = pid == s.electron_id ? "11" : "-11";
        if (hp_.scalars.action_combined_brems != invalid_id)
            continue;  // single-element materials only: nothing to select
        build(model_seltzer_berger, pid, "model." + pdg + ".e_brems.e_brems_sb");
        build(model_rel_brems, pid, "model." + pdg + ".e_brems.e_brems_lpm");
    }
    hp_.scalars.element_tables = this->add_ints(index);
}

//---------------------------------------------------------------------------//
// XORWOW jump polynomials
//---------------------------------------------------------------------------//
// Polynomials over GF(2) of degree below 192, bit m of the three 64-bit
// words holding the coefficient of z^m. The method (jump ahead by
// g(z) = z^d mod p(z), p the characteristic polynomial of the transition) is
// Haramoto et al. 2008, "Efficient jump ahead for F2-linear random number
// generators", which the reference cites (XorwowRngEngine.hh:38-52); the
// polynomials are computed here from the transition itself.
using GF2Poly = std::array<std::uint64_t, 3>;

bool gf2_bit(GF2Poly const& a, int m)
{
    return (a[m >> 6] >> (m & 63)) & 1u;
}

//! Characteristic polynomial of XORWOW's transition by Berlekamp-Massey over
//! 400 output bits (bit 0 of the last xor word after each transition). The
//! transition has period 2^160 - 1, so its characteristic polynomial is
//! primitive and is the minimal polynomial of this sequence.
GF2Poly xorwow_charpoly()
{
    std::uint32_t x[5] = {0x12345678u, 0x9abcdef0u, 0x0fedcba9u, 0x87654321u, 0x13579bdfu};
    constexpr int n = 400;
    std::vector<int> u(n);
    for (int i = 0; i < n; ++i)
    {
        xorwow_transition(x);
        u[i] = static_cast<int>(x[4] & 1u);
    }
    // Connection polynomial c: u[i] = sum_{j=1..len} c[j] u[i-j]
    std::vector<int> c(n + 1, 0), b(n + 1, 0);
    c[0] = b[0] = 1;
    int len = 0, shift = 1;
    for (int i = 0; i < n; ++i)
    {
        int d = u[i];
        for (int j = 1; j <= len; ++j)
            d ^= c[j] & u[i - j];
        if (!d)
        {
            ++shift;
            continue;
        }
        std::vector<int> const prev = c;
        for (int j = 0; j + shift <= n; ++j)
            c[j + shift] ^= b[j];
        if (2 * len <= i)
        {
            len = i + 1 - len;
            b = prev;
            shift = 1;
        }
        else
        {
            ++shift;
        }
    }
    if (len != 160)
        throw std::runtime_error("XORWOW characteristic polynomial has the wrong degree");
    // p(z) = z^160 + c1 z^159 + ... + c160: the reciprocal of c
    GF2Poly p{0, 0, 0};
    for (int j = 0; j <= len; ++j)
    {
        if (c[j])
            p[(len - j) >> 6] |= std::uint64_t(1) << ((len - j) & 63);
    }
    return p;
}

//! a z mod p, for deg a < 160
GF2Poly gf2_mul_z(GF2Poly a, GF2Poly const& p)
{
    a[2] = (a[2] << 1) | (a[1] >> 63);
    a[1] = (a[1] << 1) | (a[0] >> 63);
    a[0] <<= 1;
    if (gf2_bit(a, 160))
    {
        for (int k = 0; k < 3; ++k)
            a[k] ^= p[k];
    }
    return a;
}

//! a b mod p, by Horner's rule over the coefficients of b
GF2Poly gf2_mul_mod(GF2Poly const& a, GF2Poly const& b, GF2Poly const& p)
{
    GF2Poly r{0, 0, 0};
    for (int m = 159; m >= 0; --m)
    {
        r = gf2_mul_z(r, p);
        if (gf2_bit(b, m))
        {
            for (int k = 0; k < 3; ++k)
                r[k] ^= a[k];
        }
    }
    return r;
}

//! The five 32-bit words of a polynomial of degree below 160, low first
void store_jump_poly(GF2Poly const& g, std::uint32_t* out)
{
    for (int w = 0; w < 5; ++w)
        out[w] = static_cast<std::uint32_t>(g[w >> 1] >> (32 * (w & 1)));
}

//! Jump polynomials z^(4^i) and z^(4^i 2^67) mod p(z), i < 32, with the
//! first six checked against 4^i direct transitions
std::vector<std::uint32_t> make_xorwow_jump_polys()
{
    GF2Poly const p = xorwow_charpoly();
    std::vector<std::uint32_t> table(2 * 32 * 5);
    auto fill = [&](GF2Poly g, std::uint32_t* out) {
        for (int i = 0; i < 32; ++i)
        {
            store_jump_poly(g, out + 5 * i);
            g = gf2_mul_mod(g, g, p);
            g = gf2_mul_mod(g, g, p);
        }
    };
    GF2Poly const z{2, 0, 0};
    fill(z, table.data());
    GF2Poly sub = z;
    for (int k = 0; k < 67; ++k)
        sub = gf2_mul_mod(sub, sub, p);
    fill(sub, table.data() + 32 * 5);
    for (int i = 0; i < 6; ++i)
    {
        std::uint32_t a[5] = {1u, 2u, 3u, 4u, 5u};
        std::uint32_t b[5] = {1u, 2u, 3u, 4u, 5u};
        xorwow_apply_poly(table.data() + 5 * i, a);
        for (long n = 0; n < (1L << (2 * i)); ++n)
            xorwow_transition(b);
        for (int k = 0; k < 5; ++k)
        {
            if (a[k] != b[k])
                throw std::runtime_error("XORWOW jump polynomial check failed");
        }
    }
    return table;
}

HostParams Builder::build()
{
    if (kv_.s("format") != "gbx-physics-1")
        throw std::runtime_error("unsupported physics file format");
    this->build_actions();
    this->build_particles();
    this->build_materials();
    this->build_physics();
    this->build_models();
    this->build_element_tables();
    this->build_msc_field();
    this->build_geometry();
    hp_.rng_jump = make_xorwow_jump_polys();
    hp_.scalars.rng_per_track = opts_.rng_per_track;
    hp_.scalars.reentrant_looping = opts_.reentrant_looping;
    hp_.scalars.event_tallies = opts_.event_tallies;
    for (auto const& b : geo_.boxes)
    {
        if (b.material >= hp_.materials.size())
            throw std::runtime_error("box material out of range");
    }
    for (auto const& sh : geo_.shells)
    {
        if (sh.material >= hp_.materials.size())
            throw std::runtime_error("shell material out of range");
    }
    return std::move(hp_);
}

}  // namespace

//---------------------------------------------------------------------------//
GeometrySpec make_calorimeter_geometry(int num_layers,
                                       double absorber,
                                       double gap,
                                       double half_xy)
{
    GeometrySpec g;
    g.name = "calo";
    double const pitch = absorber + gap;
    g.world_lo[0] = g.world_lo[1] = -30;
    g.world_hi[0] = g.world_hi[1] = 30;
    g.world_lo[2] = -10;
    g.world_hi[2] = 50;
    g.background_material = 0;
    for (int k = 0; k < num_layers; ++k)
    {
        double z0 = k * pitch;
        double z1 = z0 + absorber;
        double z2 = (k + 1) * pitch;
        BoxSpec pb{"pb_" + std::to_string(k),
                   {-half_xy, -half_xy, z0},
                   {half_xy, half_xy, z1},
                   1};
        BoxSpec ar{"lar_" + std::to_string(k),
                   {-half_xy, -half_xy, z1},
                   {half_xy, half_xy, z2},
                   2};
        g.boxes.push_back(pb);
        g.boxes.push_back(ar);
    }
    return g;
}

GeometrySpec make_cms_geometry()
{
    GeometrySpec g;
    g.name = "cms";
    g.world_lo[0] = g.world_lo[1] = -310;
    g.world_hi[0] = g.world_hi[1] = 310;
    g.world_lo[2] = -320;
    g.world_hi[2] = 320;
    g.background_material = 0;
    // Silicon tracker: 10 layers of 0.3 mm, inner radii evenly from 4 to 110
    constexpr int num_si = 10;
    for (int k = 0; k < num_si; ++k)
    {
        double r = 4.0 + k * (110.0 - 4.0) / (num_si - 1);
        g.shells.push_back({"si_" + std::to_string(k), r, r + 0.03, -270, 270, 1});
    }
    // Electromagnetic calorimeter: PbWO4 crystals
    g.shells.push_back({"ecal", 129, 152, -300, 300, 2});
    // Hadron calorimeter: 17 brass + scintillator pairs between 180 and 295
    constexpr int num_hcal = 17;
    double const pitch = (295.0 - 180.0) / num_hcal;
    for (int k = 0; k < num_hcal; ++k)
    {
        double r = 180.0 + k * pitch;
        g.shells.push_back({"brass_" + std::to_string(k), r, r + 5.0, -300, 300, 3});
        g.shells.push_back(
            {"scint_" + std::to_string(k), r + 5.0, r + 5.4, -300, 300, 4});
    }
    return g;
}

GeometrySpec read_geometry_file(std::string const& path)
{
    std::ifstream in(path);
    if (!in)
        throw std::runtime_error("cannot open geometry file '" + path + "'");
    GeometrySpec g;
    g.name = path;
    g.background_material = 0;
    bool have_world = false;
    std::string line;
    int lineno = 0;
    while (std::getline(in, line))
    {
        ++lineno;
        auto hash = line.find('#');
        if (hash != std::string::npos)
            line.erase(hash);
        std::istringstream ls(line);
        std::string kind;
        if (!(ls >> kind))
            continue;
        auto fail = [&](char const* what) {
            throw std::runtime_error(path + ":" + std::to_string(lineno) + ": " + what);
        };
        if (kind == "gbx-geometry")
        {
            int version = 0;
            if (!(ls >> version) || version != 1)
                fail("unsupported geometry file version");
        }
        else if (kind == "world")
        {
            for (double& v : g.world_lo)
                ls >> v;
            for (double& v : g.world_hi)
                ls >> v;
            if (!ls)
                fail("world needs lo_x lo_y lo_z hi_x hi_y hi_z");
            have_world = true;
        }
        else if (kind == "background")
        {
            if (!(ls >> g.background_material))
                fail("background needs a material index");
        }
        else if (kind == "box")
        {
            BoxSpec b;
            ls >> b.label >> b.material;
            for (double& v : b.lo)
                ls >> v;
            for (double& v : b.hi)
                ls >> v;
            if (!ls)
                fail("box needs label material lo_x lo_y lo_z hi_x hi_y hi_z");
            for (int ax = 0; ax < 3; ++ax)
            {
                if (!(b.lo[ax] < b.hi[ax]))
                    fail("box with an empty extent");
            }
            g.boxes.push_back(b);
        }
        else if (kind == "shell")
        {
            ShellSpec sh;
            if (!(ls >> sh.label >> sh.material >> sh.r_in >> sh.r_out >> sh.z_lo >> sh.z_hi))
                fail("shell needs label material r_in r_out z_lo z_hi");
            g.shells.push_back(sh);
        }
        else
        {
            fail("unknown record (expected world, background, box or shell)");
        }
    }
    if (!have_world)
        throw std::runtime_error(path + ": no world box");
    if (g.boxes.empty() == g.shells.empty())
        throw std::runtime_error(path + ": a geometry holds either boxes or shells");
    return g;
}

GeometrySpec make_geometry(std::string const& name)
{
    if (name == "calo")
        return make_calorimeter_geometry();
    if (name == "cms")
        return make_cms_geometry();
    if (std::ifstream(name))
        return read_geometry_file(name);
    throw std::runtime_error("unknown geometry '" + name
                             + "' (neither 'calo', 'cms' nor a geometry file)");
}

HostParams build_params(std::string const& physics_path,
                        GeometrySpec const& geo,
                        ParamsOptions const& opts)
{
    KvFile kv(physics_path);
    Builder b(kv, geo, opts);
    return b.build();
}

ParamsData make_host_view(HostParams const& hp)
{
    ParamsData p = hp.scalars;
    p.reals = hp.reals.data();
    p.ints = hp.ints.data();
    p.particles = hp.particles.data();
    p.materials = hp.materials.data();
    p.elements = hp.elements.data();
    p.fluct = hp.fluct.data();
    p.cutoff_energy = hp.cutoffs.data();
    p.process_groups = hp.groups.data();
    p.grids = hp.grids.data();
    p.livermore_elements = hp.lv_elements.data();
    p.livermore_shells = hp.lv_shells.data();
    p.sb_tables = hp.sb_tables.data();
    p.rb_elements = hp.rb_elements.data();
    p.msc.material = hp.msc_materials.data();
    p.msc.par_mat = hp.msc_par_mat.data();
    p.looping = hp.looping.data();
    p.rng_jump = hp.rng_jump.data();
    p.rzmap = hp.rzmap.empty() ? nullptr : &hp.rzmap_desc;
    p.geo.surfaces = hp.surfaces.data();
    p.geo.volumes = hp.volumes.data();
    p.geo.neighbor_offset = hp.neighbor_offset.data();
    p.geo.neighbors = hp.neighbors.data();
    p.geo.sorted_surfaces = hp.sorted_surfaces.data();
    p.geo.sorted_key = hp.sorted_key.data();
    p.geo.volume_material = hp.volume_material.data();
    p.geo.volume_detector = hp.volume_detector.data();
    return p;
}

}  // namespace gbx
