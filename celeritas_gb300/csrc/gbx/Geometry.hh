// Navigation through volumes bounded by axis-aligned planes and z-axis
// cylinders inside an implicit background volume and a world box (the
// sampling-calorimeter and CMS-like geometry classes).
//
// Semantics follow ORANGE's single-level simple unit:
// - sense of a point w.r.t. a surface is "outside" when the surface function
//   is >= 0: pos - plane for planes, x^2 + y^2 - r^2 for z cylinders
//   (src/orange/OrangeTypes.hh:412-424, src/orange/surf/CylCentered.hh);
// - a volume's logic is the conjunction of its face senses
//   (src/orange/univ/detail/LogicEvaluator.hh);
// - distance to a plane is (plane - pos) / dir, kept if positive and not on
//   the current surface (src/orange/surf/PlaneAligned.hh); a cylinder's
//   distances are the positive roots of its quadratic, with the on-surface
//   (c = 0) form on the current surface
//   (src/orange/surf/detail/QuadraticSolver.hh);
// - a volume takes the first minimum over its faces' intersections
//   (src/orange/univ/SimpleUnitTracker.hh:271-330);
// - the background volume accepts the first crossing, by increasing
//   (distance, surface), whose bumped point lies inside a neighbor volume
//   (SimpleUnitTracker::background_intersect);
// - crossing a surface flips the sense and locates the new volume among the
//   surface's neighbors with the crossed face's sense forced
//   (SimpleUnitTracker::cross_boundary, OrangeTrackView.hh:662-787);
// - moving uses axpy with fma (src/corecel/math/ArrayUtils.hh:78-85).
//
// The volume search used when a surface has many neighbors (the reference
// uses a bounding-interval hierarchy) is a binary search over the layer
// planes for boxes stacked along z, or a scan over the volumes; either
// selects the same volume because volumes do not overlap.
#pragma once

#include "Data.hh"

namespace gbx
{
struct Propagation
{
    double distance;
    bool boundary;
    bool looping;
};

//! First index in [lo, hi) whose sorted key is not below x (hi if none)
GBX_FORCEINLINE size_type key_lower_bound(float const* key,
                                          size_type lo,
                                          size_type hi,
                                          float x)
{
    while (lo < hi)
    {
        size_type const mid = lo + (hi - lo) / 2;
        if (key[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

//! First index in [lo, hi) whose sorted key is above x (hi if none)
GBX_FORCEINLINE size_type key_upper_bound(float const* key,
                                          size_type lo,
                                          size_type hi,
                                          float x)
{
    while (lo < hi)
    {
        size_type const mid = lo + (hi - lo) / 2;
        if (!(x < key[mid]))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

class GeoTrackView
{
  public:
    GBX_FORCEINLINE GeoTrackView(GeoParams const& params,
                                 StateData const& state,
                                 size_type slot)
        : p_(params), s_(state), slot_(slot)
    {
    }

    //// ACCESSORS ////
    GBX_FORCEINLINE Real3 pos() const
    {
        return {s_.pos[0][slot_], s_.pos[1][slot_], s_.pos[2][slot_]};
    }
    GBX_FORCEINLINE Real3 dir() const
    {
        return {s_.dir[0][slot_], s_.dir[1][slot_], s_.dir[2][slot_]};
    }
    GBX_FORCEINLINE size_type volume() const { return s_.volume[slot_]; }
    GBX_FORCEINLINE bool is_outside() const
    {
        return s_.volume[slot_] == p_.exterior;
    }
    GBX_FORCEINLINE bool is_on_boundary() const
    {
        return s_.surface[slot_] != invalid_id;
    }
    GBX_FORCEINLINE bool failed() const { return s_.geo_failed[slot_] != 0; }

    //// INITIALIZATION ////
    //! Locate a new track from scratch (OrangeTrackView operator=(Initializer))
    GBX_FUNCTION void initialize(Real3 const& pos, Real3 const& dir)
    {
        this->set_pos(pos);
        this->set_dir_raw(dir);
        bool on_surface = false;
        size_type vol
            = this->find_volume_at(pos, invalid_id, invalid_id, &on_surface);
        std::uint8_t failed = 0;
        if (on_surface)
        {
            failed = 1;
            vol = p_.exterior;
        }
        s_.volume[slot_] = vol;
        s_.geo_failed[slot_] = failed;
        s_.boundary[slot_] = boundary_exiting;
        s_.surface[slot_] = invalid_id;
        s_.surface_sense[slot_] = 0;
        s_.next_step[slot_] = 0;
        s_.next_surface[slot_] = invalid_id;
    }

    //! Copy another track's geometry state with a new direction
    //! (OrangeTrackView operator=(DetailedInitializer))
    GBX_FUNCTION void copy_from(size_type other, Real3 const& dir)
    {
        if (other != slot_)
        {
            s_.volume[slot_] = s_.volume[other];
            s_.surface[slot_] = s_.surface[other];
            s_.surface_sense[slot_] = s_.surface_sense[other];
            s_.boundary[slot_] = s_.boundary[other];
            for (int i = 0; i < 3; ++i)
            {
                s_.pos[i][slot_] = s_.pos[i][other];
            }
        }
        s_.geo_failed[slot_] = 0;
        s_.next_step[slot_] = 0;
        s_.next_surface[slot_] = invalid_id;
        this->set_dir_raw(dir);
    }

    //// NAVIGATION ////
    GBX_FUNCTION Propagation find_next_step(double max_step);
    GBX_FUNCTION void move_to_boundary();
    GBX_FUNCTION void move_internal(double dist);
    //! Move within the current volume to a nearby point
    GBX_FORCEINLINE void move_internal_to(Real3 const& pos)
    {
        this->set_pos(pos);
        s_.surface[slot_] = invalid_id;
        s_.next_step[slot_] = 0;
        s_.next_surface[slot_] = invalid_id;
    }
    GBX_FUNCTION void cross_boundary();
    //! Whether find_next_step would solve the surfaces: the track is
    //! neither on a boundary nor flagged to re-enter its volume
    GBX_FORCEINLINE bool is_clear_of_boundary() const
    {
        return s_.surface[slot_] == invalid_id
               && s_.boundary[slot_] != boundary_reentrant;
    }
    //! find_next_step's result and state for a segment of length max_step
    //! that reaches no surface (the caller has a surface-free ball around it)
    GBX_FORCEINLINE Propagation no_crossing(double max_step)
    {
        s_.next_step[slot_] = max_step;
        s_.next_surface[slot_] = invalid_id;
        s_.next_sense[slot_] = 0;
        return {max_step, false, false};
    }
    GBX_FUNCTION void set_dir(Real3 const& newdir);
    GBX_FUNCTION double find_safety() const;

  private:
    GeoParams const& p_;
    StateData const& s_;
    size_type slot_;

    GBX_FORCEINLINE void set_pos(Real3 const& v)
    {
        s_.pos[0][slot_] = v.x;
        s_.pos[1][slot_] = v.y;
        s_.pos[2][slot_] = v.z;
    }
    GBX_FORCEINLINE void set_dir_raw(Real3 const& v)
    {
        s_.dir[0][slot_] = v.x;
        s_.dir[1][slot_] = v.y;
        s_.dir[2][slot_] = v.z;
    }

    //! True if the point is on the "outside" (non-negative) side of a surface
    static GBX_FORCEINLINE bool sense_outside(double q) { return !(q < 0); }

    //! Surface function at a point: its sign is the sense
    GBX_FORCEINLINE double surface_q(size_type surf, Real3 const& pos) const
    {
        SurfaceRecord const& sr = p_.surfaces[surf];
        if (sr.type == surf_czc)
            return ipow<2>(pos.x) + ipow<2>(pos.y) - sr.value;
        return pos[sr.type] - sr.value;
    }

    //! Positive distances to a surface along dir (+inf where none). Surfaces
    //! whose nearest point is farther than max_dist are skipped without
    //! solving: every distance along the ray is at least that far, so the
    //! caller's "d <= max_dist" test would reject them anyway.
    GBX_FUNCTION void intersect(size_type surf,
                                Real3 const& pos,
                                Real3 const& dir,
                                bool on_surface,
                                double* dist,
                                double max_dist = INFINITY) const
    {
        dist[0] = dist[1] = INFINITY;
        SurfaceRecord const& sr = p_.surfaces[surf];
        if (sr.type != surf_czc)
        {
            if (on_surface)
                return;
            // |d| = |plane - pos| / |dir_axis| >= |plane - pos|, also after
            // rounding since |dir_axis| <= 1
            if (!(std::fabs(sr.value - pos[sr.type]) <= max_dist))
                return;
            double const n_dir = dir[sr.type];
            if (n_dir != 0)
            {
                double const d = (sr.value - pos[sr.type]) / n_dir;
                if (d > 0)
                    dist[0] = d;
            }
            return;
        }
        if (!on_surface && max_dist < INFINITY)
        {
            // The radial distance |r - R| bounds the distance along any ray;
            // skip the cylinder unless r lies within max_dist of R. The test
            // runs in FP32 (the FP64 pipe is the scarce one) with a margin of
            // 1e-5 (R + max_dist) + 1e-6 cm: FP32 rounding of r^2 and of the
            // bounds is below 1e-6 relative, and the rounding of the
            // quadratic's FP64 roots far below that, so a skipped cylinder
            // has no root within max_dist and the hit is unchanged. Distances
            // beyond FP32 range give infinite bounds: nothing is skipped.
            float const xf = static_cast<float>(pos.x);
            float const yf = static_cast<float>(pos.y);
            float const r2 = xf * xf + yf * yf;
            float const df = static_cast<float>(max_dist);
            float const margin = 1e-5f * (sr.radius + df) + 1e-6f;
            float const hi = sr.radius + df + margin;
            float const lo = sr.radius - df - margin;
            if (r2 > hi * hi || (lo > 0 && r2 < lo * lo))
                return;
        }
        // 1 - (dir . z)^2; no intersection when traveling along the axis
        double const a = 1 - ipow<2>(dir.z);
        constexpr double sqrt_quadratic = 1e-5;
        if (a < ipow<2>(sqrt_quadratic))
            return;
        double const half_b = dir.x * pos.x + dir.y * pos.y;
        double const a_inv = 1 / a;
        double const hba = half_b * a_inv;
        if (on_surface)
        {
            double const r = -2 * hba;
            if (r > 0)
                dist[0] = r;
            return;
        }
        double const c = (ipow<2>(pos.x) + ipow<2>(pos.y) - sr.value) * a_inv;
        double const b2_4 = ipow<2>(hba);
        if (b2_4 > c)
        {
            double const t2 = std::sqrt(b2_4 - c);
            double const r0 = -hba - t2;
            double const r1 = -hba + t2;
            if (r1 > 0)
            {
                dist[1] = r1;
                if (r0 > 0)
                    dist[0] = r0;
            }
        }
        else if (b2_4 == c)
        {
            double const r0 = -hba;
            if (r0 > 0)
                dist[0] = r0;
        }
    }

    //! Accepted background crossing with the least (distance, surface ID)
    struct Crossing
    {
        size_type surf;  //!< invalid_id while none is accepted
        double dist;  //!< Its distance (the step limit while none)
        std::int8_t sense;  //!< Sense of the crossed surface in the new volume
    };
    //! Largest distance at which a crossing can still replace the current
    //! one (at equal distance the lower surface ID wins)
    static GBX_FORCEINLINE double crossing_limit(Crossing const& hit)
    {
        return hit.dist;
    }
    GBX_FUNCTION void consider_crossing(size_type surf,
                                        double d,
                                        Real3 const& pos,
                                        Real3 const& dir,
                                        double bump,
                                        double max_step,
                                        Crossing* hit) const;
    GBX_FUNCTION void background_crossing(Real3 const& pos,
                                          Real3 const& dir,
                                          size_type cur_surf,
                                          double max_step,
                                          Crossing* hit) const;

    //! Distance from a point to a surface (for the safety): the nearest
    //! intersection along the surface normal pointing toward the surface
    //! (CalcSafetyDistance, src/orange/univ/detail/SurfaceFunctors.hh)
    GBX_FUNCTION double surface_safety(size_type surf, Real3 const& pos) const
    {
        SurfaceRecord const& sr = p_.surfaces[surf];
        if (sr.type != surf_czc)
            return std::fabs(pos[sr.type] - sr.value);
        if constexpr (sizeof(real_type) < sizeof(double))
        {
            // Mixed build: the same distance |r - R| from the radius, about
            // a third of the FP64 instructions of the normal-direction solve
            // below (equal to it within FP64 rounding of the radii), with the
            // same infinite safety on the axis
            double const rsq = ipow<2>(pos.x) + ipow<2>(pos.y);
            if (!(rsq > 0))
                return INFINITY;
            double const q = rsq - sr.value;
            if (q == 0)
                return 0;
            return std::fabs(std::sqrt(rsq) - sr.radius_d);
        }
        Real3 n = make_unit_vector(Real3{pos.x, pos.y, 0});
        if (std::isnan(n.x))
        {
            // On the axis: the cylinder is a long way off
            return INFINITY;
        }
        double const q = this->surface_q(surf, pos);
        if (q > 0)
        {
            n = {-n.x, -n.y, -n.z};
        }
        else if (q == 0)
        {
            return 0;
        }
        double d[2];
        this->intersect(surf, pos, n, false, d);
        return min_of(d[0], d[1]);
    }

    //! Evaluate the inside logic of a volume at 'pos'. A face whose
    //! surface equals 'forced' takes the given sense. Sets *on_surface if
    //! any unforced face evaluates exactly on its surface.
    GBX_FUNCTION bool volume_logic(VolumeRecord const& vol,
                                   Real3 const& pos,
                                   size_type forced,
                                   bool forced_outside,
                                   bool* on_surface) const
    {
        bool inside = true;
        for (size_type f = 0; f < vol.num_faces; ++f)
        {
            bool s;
            if (vol.faces[f] == forced)
            {
                s = forced_outside;
            }
            else
            {
                double q = this->surface_q(vol.faces[f], pos);
                s = sense_outside(q);
                if (q == 0 && on_surface)
                {
                    *on_surface = true;
                }
            }
            inside = inside && (vol.inside_sense[f] > 0 ? s : !s);
            // Without an on-surface report the remaining faces cannot
            // change the answer
            if (!inside && !on_surface)
                return false;
        }
        return inside;
    }

    //! Exterior volume logic: not inside the world box
    GBX_FUNCTION bool exterior_inside(Real3 const& pos,
                                      size_type forced,
                                      bool forced_outside,
                                      bool* on_surface) const
    {
        VolumeRecord world;
        for (int f = 0; f < 6; ++f)
        {
            world.faces[f] = p_.world_faces[f];
            world.inside_sense[f] = p_.world_sense[f];
        }
        world.num_faces = 6;
        return !this->volume_logic(world, pos, forced, forced_outside, on_surface);
    }

    GBX_FUNCTION bool volume_inside(size_type vol,
                                    Real3 const& pos,
                                    size_type forced,
                                    bool forced_outside,
                                    bool* on_surface) const
    {
        if (vol == p_.exterior)
        {
            return this->exterior_inside(pos, forced, forced_outside, on_surface);
        }
        return this->volume_logic(
            p_.volumes[vol], pos, forced, forced_outside, on_surface);
    }

    //! Locate the volume containing a point among all volumes (the
    //! reference's BIH search), skipping 'exclude'; background if none.
    GBX_FUNCTION size_type find_volume_at(Real3 const& pos,
                                          size_type exclude,
                                          size_type forced,
                                          bool* on_surface,
                                          bool forced_outside = false) const;
};

//---------------------------------------------------------------------------//
GBX_FUNCTION size_type GeoTrackView::find_volume_at(Real3 const& pos,
                                                    size_type exclude,
                                                    size_type forced,
                                                    bool* on_surface,
                                                    bool forced_outside) const
{
    // Exterior first: outside the world box
    // Faces are evaluated to the last only when the caller wants to know
    // whether the point lies on one
    if (exclude != p_.exterior)
    {
        bool on = false;
        if (this->exterior_inside(pos, forced, forced_outside, on_surface ? &on : nullptr))
        {
            if (on_surface)
                *on_surface = on;
            return p_.exterior;
        }
    }
    if (p_.locate == locate_scan)
    {
        for (size_type cand = 1; cand < p_.background; ++cand)
        {
            if (cand == exclude)
                continue;
            bool on = false;
            if (this->volume_logic(p_.volumes[cand],
                                   pos,
                                   forced,
                                   forced_outside,
                                   on_surface ? &on : nullptr))
            {
                if (on_surface)
                    *on_surface = on;
                return cand;
            }
        }
        return p_.background;
    }
    // Candidate box volumes: binary search along z over the volumes' lower
    // planes (boxes are sorted by increasing lower plane)
    double const x = pos.z;
    // Boxes occupy ids [1, background); find last box with lower <= x
    size_type lo = 1, hi = p_.background;  // search in [lo, hi)
    while (lo < hi)
    {
        size_type mid = lo + (hi - lo) / 2;
        double lower = p_.surfaces[p_.volumes[mid].faces[4]].value;
        if (lower <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    // lo - 1 is the last box whose lower plane is <= x; also test the one
    // below in case the point sits exactly on a shared plane
    for (int k = 0; k < 2; ++k)
    {
        if (lo < 2 + static_cast<size_type>(k))
            break;
        size_type cand = lo - 1 - k;
        if (cand == exclude)
            continue;
        bool on = false;
        if (this->volume_logic(
                p_.volumes[cand], pos, forced, forced_outside, on_surface ? &on : nullptr))
        {
            if (on_surface)
                *on_surface = on;
            return cand;
        }
    }
    return p_.background;
}

//---------------------------------------------------------------------------//
GBX_FUNCTION Propagation GeoTrackView::find_next_step(double max_step)
{
    Propagation result{max_step, false, false};
    if (s_.boundary[slot_] == boundary_reentrant)
    {
        s_.next_step[slot_] = 0;
        s_.next_surface[slot_] = s_.surface[slot_];
        s_.next_sense[slot_] = s_.surface_sense[slot_];
        return {0, true, false};
    }
    Real3 const pos = this->pos();
    Real3 const dir = this->dir();
    size_type const vol = s_.volume[slot_];
    size_type const cur_surf = s_.surface[slot_];

    size_type hit_surf = invalid_id;
    double hit_dist = max_step;
    std::int8_t hit_sense = 0;

    if (vol != p_.background)
    {
        // Volume of face conjunctions: first minimum over the faces'
        // intersections in face order
        VolumeRecord const& v = p_.volumes[vol];
        double best = INFINITY;
        size_type best_face = invalid_id;
        for (size_type f = 0; f < v.num_faces; ++f)
        {
            double d[2];
            this->intersect(v.faces[f], pos, dir, v.faces[f] == cur_surf, d, max_step);
            for (int k = 0; k < 2; ++k)
            {
                if (d[k] <= max_step && d[k] < best)
                {
                    best = d[k];
                    best_face = f;
                }
            }
        }
        if (best_face != invalid_id)
        {
            hit_surf = v.faces[best_face];
            hit_dist = best;
            if (hit_surf == cur_surf)
            {
                hit_sense = s_.surface_sense[slot_];
            }
            else
            {
                hit_sense = sense_outside(this->surface_q(hit_surf, pos)) ? 1 : -1;
            }
        }
    }
    else
    {
        Crossing hit{invalid_id, max_step, 0};
        this->background_crossing(pos, dir, cur_surf, max_step, &hit);
        hit_surf = hit.surf;
        hit_dist = hit.dist;
        hit_sense = hit.sense;
    }

    s_.next_step[slot_] = hit_dist;
    s_.next_surface[slot_] = hit_surf;
    s_.next_sense[slot_] = hit_sense;
    result.distance = hit_dist;
    result.boundary = (hit_surf != invalid_id);
    return result;
}

//! Test one background crossing: a candidate at distance d on surface surf
//! that would improve the current crossing is accepted if the point bumped
//! past it lies inside a volume neighboring the surface
GBX_FUNCTION void GeoTrackView::consider_crossing(size_type surf,
                                                  double d,
                                                  Real3 const& pos,
                                                  Real3 const& dir,
                                                  double bump,
                                                  double max_step,
                                                  Crossing* hit) const
{
    if (!(d <= max_step))
        return;
    if (hit->surf != invalid_id
        && !(d < hit->dist || (d == hit->dist && surf < hit->surf)))
    {
        return;
    }
    Real3 bumped = pos;
    axpy(d + bump, dir, &bumped);
    // Neighbors of this surface
    size_type nbeg = p_.neighbor_offset[surf];
    size_type nend = p_.neighbor_offset[surf + 1];
    bool found = false;
    bool found_outside = false;
    if (nend - nbeg >= 3)
    {
        // Many neighbors: locate by position (non-overlapping)
        size_type v = this->find_volume_at(bumped, invalid_id, invalid_id, nullptr);
        if (v != p_.background && v != p_.exterior)
        {
            found = true;
            // Sense of the crossed surface evaluated at the bumped point
            // inside the new volume, flipped
            found_outside = !sense_outside(this->surface_q(surf, bumped));
        }
    }
    else
    {
        for (size_type n = nbeg; n < nend; ++n)
        {
            size_type v = p_.neighbors[n];
            if (this->volume_inside(v, bumped, invalid_id, false, nullptr))
            {
                found = true;
                found_outside = !sense_outside(this->surface_q(surf, bumped));
                break;
            }
        }
    }
    if (found)
    {
        hit->surf = surf;
        hit->dist = d;
        hit->sense = found_outside ? 1 : -1;
    }
}

//! Next boundary crossing of a track in the implicit background.
//!
//! The reference visits crossings by increasing (distance, surface ID) and
//! accepts the first whose bumped point lies inside a neighboring volume
//! (SimpleUnitTracker::background_intersect,
//! src/orange/univ/SimpleUnitTracker.hh:572-645).
//! Acceptance depends on that crossing alone, so the result is the least
//! (distance, surface ID) over accepted crossings, whatever order they are
//! tested in; a crossing is tested only if it would improve the current one.
//!
//! Instead of solving every surface, the search walks the surfaces of each
//! kind in the order the ray meets them and stops at the first whose
//! distance exceeds the current crossing's. Each walk's distances are
//! computed exactly as the per-surface solve computes them, and they are
//! monotone along the walk in floating point, not only in exact arithmetic:
//! - planes normal to axis k, moving toward +k: d = (v - x) / n grows with
//!   the plane's value v (IEEE subtraction and division are monotone);
//! - z cylinders of squared radius v: the solve forms c = (x^2 + y^2 - v)/a,
//!   compares hba^2 with c and takes t = sqrt(hba^2 - c); c falls as v
//!   grows, so whether the ray reaches the cylinder, the far root
//!   -hba + t (growing with v) and the near root -hba - t (falling with v)
//!   are all monotone. Near roots are walked downward from the track's
//!   radius, far roots upward from just below it (a reached cylinder well
//!   inside the track's radius has both roots taken by the downward walk).
//! Index bounds from the FP32 keys only ever start a walk earlier than
//! needed (rounding to FP32 is monotone too), and an FP32 radial bound |r -
//! R| stops a cylinder walk only where every root is beyond the limit, with
//! the same margin as the per-surface reachability test. The result is
//! therefore the crossing a solve of every surface would give.
GBX_FUNCTION void GeoTrackView::background_crossing(Real3 const& pos,
                                                    Real3 const& dir,
                                                    size_type cur_surf,
                                                    double max_step,
                                                    Crossing* hit) const
{
    double bump = p_.tol_abs;
    for (int i = 0; i < 3; ++i)
    {
        bump = max_of(bump, p_.tol_rel * std::fabs(pos[i]));
    }
#ifdef GBX_GEO_SCAN_BACKGROUND
    // Every surface in ID order (the CPU oracle's restatement, compiled
    // only there to check the ordered walks below)
    for (size_type surf = 0; surf < p_.num_surfaces; ++surf)
    {
        double dd[2];
        this->intersect(surf, pos, dir, surf == cur_surf, dd, max_step);
        for (int k = 0; k < 2; ++k)
            this->consider_crossing(surf, dd[k], pos, dir, bump, max_step, hit);
    }
    return;
#endif
    size_type const* sorted = p_.sorted_surfaces;
    float const* key = p_.sorted_key;

    // The surface the track is on: its crossing comes from the on-surface
    // solve
    if (cur_surf != invalid_id)
    {
        double dd[2];
        this->intersect(cur_surf, pos, dir, true, dd);
        for (int k = 0; k < 2; ++k)
            this->consider_crossing(cur_surf, dd[k], pos, dir, bump, max_step, hit);
    }

    // Z cylinders first: in a barrel of shells they usually hold the nearest
    // crossing, which then bounds the plane walks below, so that fewer
    // plane candidates need the acceptance test (a plane shared by many
    // shells locates the bumped point among all volumes). The per-surface
    // solve finds no cylinder crossing when traveling along the axis.
    size_type const cbeg = p_.sorted_offset[surf_czc];
    size_type const cend = p_.sorted_offset[surf_czc + 1];
    constexpr double sqrt_quadratic = 1e-5;
    if (cbeg < cend && !(1 - ipow<2>(dir.z) < ipow<2>(sqrt_quadratic)))
    {
        float const xf = static_cast<float>(pos.x);
        float const yf = static_cast<float>(pos.y);
        float const rf = std::sqrt(xf * xf + yf * yf);
        auto radial_margin = [](float radius, float limit) {
            return 1e-5f * (radius + limit) + 1e-6f;
        };

        // Near roots (entering a smaller cylinder while moving inward), walked
        // down from the track's radius r: they grow as the radius falls.
        // Cylinders with keys above FP32(r) (1 + 1e-6) are outside r and have no
        // near root.
        for (size_type i = key_upper_bound(key, cbeg, cend, rf + (1e-6f * rf + 1e-20f));
             i-- > cbeg;)
        {
            size_type const surf = sorted[i];
            if (surf == cur_surf)
                continue;
            double const limit = crossing_limit(*hit);
            float const limit_f = static_cast<float>(limit);
            if (rf - key[i] - radial_margin(key[i], limit_f) > limit_f)
                break;
            double dd[2];
            this->intersect(surf, pos, dir, false, dd);
            if (dd[0] < INFINITY)
            {
                if (dd[0] > limit)
                    break;
                for (int k = 0; k < 2; ++k)
                    this->consider_crossing(surf, dd[k], pos, dir, bump, max_step, hit);
            }
            else if (!(dd[1] < INFINITY))
            {
                // Not reached, or moving outward: nor is any smaller cylinder
                break;
            }
            // Else only a far root (a cylinder at r, or just below it with a
            // near root that rounds to zero): the upward walk takes it
        }

        // Far roots, walked up from just below r: they grow with the radius.
        // Below r - 1e-4 (r + 1) a reached cylinder has a near root of at least
        // 5e-5 times its far one, so the downward walk above has taken
        // both of its roots, or stopped where both lie beyond the limit.
        float const delta = 1e-4f * (rf + 1);
        for (size_type i = key_lower_bound(key, cbeg, cend, rf - delta); i < cend; ++i)
        {
            size_type const surf = sorted[i];
            if (surf == cur_surf)
                continue;
            double const limit = crossing_limit(*hit);
            float const limit_f = static_cast<float>(limit);
            if (key[i] - rf - radial_margin(key[i], limit_f) > limit_f)
                break;
            double dd[2];
            this->intersect(surf, pos, dir, false, dd);
            double const far = (dd[1] < INFINITY) ? dd[1] : dd[0];
            if (!(far < INFINITY))
            {
                // Behind the track or not reached: a larger cylinder may be
                continue;
            }
            if (far > limit)
                break;
            for (int k = 0; k < 2; ++k)
                this->consider_crossing(surf, dd[k], pos, dir, bump, max_step, hit);
        }
    }

    // Planes of each axis, in the order the ray meets them. A plane's
    // distance |v - x| / |n| is at least |v - x| (1 - 2^-40) for a unit
    // direction rounded to FP64, which ends the walk without a division.
    for (int ax = 0; ax < 3; ++ax)
    {
        double const n = dir[ax];
        if (n == 0)
            continue;
        size_type const beg = p_.sorted_offset[ax];
        size_type const end = p_.sorted_offset[ax + 1];
        double const x = pos[ax];
        float const xf = static_cast<float>(x);
        if (n > 0)
        {
            // Planes ahead (v > x) have keys at or above FP32(x)
            for (size_type i = key_lower_bound(key, beg, end, xf); i < end; ++i)
            {
                size_type const surf = sorted[i];
                double const gap = p_.surfaces[surf].value - x;
                if (!(gap > 0) || surf == cur_surf)
                    continue;
                if (gap * (1 - 0x1p-40) > crossing_limit(*hit))
                    break;
                double const d = gap / n;
                if (d > 0)
                    this->consider_crossing(surf, d, pos, dir, bump, max_step, hit);
            }
        }
        else
        {
            // Planes behind (v < x) have keys at or below FP32(x)
            for (size_type i = key_upper_bound(key, beg, end, xf); i-- > beg;)
            {
                size_type const surf = sorted[i];
                double const gap = p_.surfaces[surf].value - x;
                if (!(gap < 0) || surf == cur_surf)
                    continue;
                if (-gap * (1 - 0x1p-40) > crossing_limit(*hit))
                    break;
                double const d = gap / n;
                if (d > 0)
                    this->consider_crossing(surf, d, pos, dir, bump, max_step, hit);
            }
        }
    }
}

GBX_FUNCTION void GeoTrackView::move_to_boundary()
{
    double const dist = s_.next_step[slot_];
    Real3 pos = this->pos();
    axpy(dist, this->dir(), &pos);
    this->set_pos(pos);
    s_.surface[slot_] = s_.next_surface[slot_];
    s_.surface_sense[slot_] = s_.next_sense[slot_];
    s_.next_step[slot_] = 0;
    s_.next_surface[slot_] = invalid_id;
}

GBX_FUNCTION void GeoTrackView::move_internal(double dist)
{
    Real3 pos = this->pos();
    axpy(dist, this->dir(), &pos);
    this->set_pos(pos);
    s_.next_step[slot_] = s_.next_step[slot_] - dist;
    s_.surface[slot_] = invalid_id;
}

GBX_FUNCTION void GeoTrackView::cross_boundary()
{
    if (s_.boundary[slot_] == boundary_reentrant)
    {
        s_.boundary[slot_] = boundary_exiting;
        return;
    }
    // Flip the sense on crossing
    std::int8_t sense = -s_.surface_sense[slot_];
    s_.surface_sense[slot_] = sense;
    s_.boundary[slot_] = boundary_exiting;

    size_type const surf = s_.surface[slot_];
    size_type const cur_vol = s_.volume[slot_];
    Real3 const pos = this->pos();
    bool const forced_outside = sense > 0;

    size_type nbeg = p_.neighbor_offset[surf];
    size_type nend = p_.neighbor_offset[surf + 1];
    size_type new_vol = invalid_id;
    if (nend - nbeg < 3)
    {
        for (size_type n = nbeg; n < nend; ++n)
        {
            size_type v = p_.neighbors[n];
            if (v == cur_vol)
                continue;
            if (this->volume_inside(v, pos, surf, forced_outside, nullptr))
            {
                new_vol = v;
                break;
            }
        }
    }
    else
    {
        new_vol = this->find_volume_at(pos, cur_vol, surf, nullptr, forced_outside);
        if (new_vol == p_.background)
            new_vol = invalid_id;
    }
    if (new_vol == invalid_id)
    {
        new_vol = p_.background;
    }
    s_.volume[slot_] = new_vol;
}

GBX_FUNCTION void GeoTrackView::set_dir(Real3 const& newdir)
{
    size_type const surf = s_.surface[slot_];
    if (surf != invalid_id)
    {
        // Sign of the direction along the surface normal: the unit axis for
        // a plane, (x, y, 0) for a z cylinder
        SurfaceRecord const& sr = p_.surfaces[surf];
        Real3 const olddir = this->dir();
        double n_new, n_old;
        if (sr.type == surf_czc)
        {
            Real3 const pos = this->pos();
            n_new = newdir.x * pos.x + newdir.y * pos.y;
            n_old = olddir.x * pos.x + olddir.y * pos.y;
        }
        else
        {
            n_new = newdir[sr.type];
            n_old = olddir[sr.type];
        }
        if ((n_new >= 0) != (n_old >= 0))
        {
            s_.boundary[slot_] = (s_.boundary[slot_] == boundary_exiting)
                                     ? boundary_reentrant
                                     : boundary_exiting;
        }
    }
    this->set_dir_raw(newdir);
    s_.next_step[slot_] = 0;
    s_.next_surface[slot_] = invalid_id;
}

GBX_FUNCTION double GeoTrackView::find_safety() const
{
    Real3 const pos = this->pos();
    size_type const vol = s_.volume[slot_];
    double result = INFINITY;
    // A cylinder's safety distance is |r - R| up to FP64 rounding (~1e-13
    // relative). Its FP32 lower bound |r - R| - 1e-5 (R + r + best) - 1e-6
    // stays below the exact value by far more than FP32 rounding (below
    // 1e-6 relative), so a cylinder whose bound exceeds the best distance so
    // far cannot lower the minimum and its FP64 solve is skipped: the result
    // is unchanged, and far cylinders cost a few FP32 operations.
    float const xf = static_cast<float>(pos.x);
    float const yf = static_cast<float>(pos.y);
    float const rf = std::sqrt(xf * xf + yf * yf);
    auto visit = [&](size_type surf) {
        SurfaceRecord const& sr = p_.surfaces[surf];
        if (sr.type == surf_czc)
        {
            float const best = static_cast<float>(result);
            float const margin = 1e-5f * (sr.radius + rf + best) + 1e-6f;
            if (std::fabs(rf - sr.radius) - margin > best)
                return;
        }
        result = min_of(result, this->surface_safety(surf, pos));
    };
    if (vol != p_.background)
    {
        VolumeRecord const& v = p_.volumes[vol];
        for (size_type f = 0; f < v.num_faces; ++f)
        {
            visit(v.faces[f]);
        }
    }
#ifdef GBX_GEO_SCAN_BACKGROUND
    else
    {
        for (size_type surf = 0; surf < p_.num_surfaces; ++surf)
            visit(surf);
    }
#else
    else
    {
        // Every surface bounds the background. Planes: the nearest on either
        // side of the point along each axis (|x - v| grows away from x;
        // keys below FP32(x) belong to planes below x)
        size_type const* sorted = p_.sorted_surfaces;
        float const* key = p_.sorted_key;
        for (int ax = 0; ax < 3; ++ax)
        {
            size_type const beg = p_.sorted_offset[ax];
            size_type const end = p_.sorted_offset[ax + 1];
            double const x = pos[ax];
            size_type const mid = key_lower_bound(key, beg, end, static_cast<float>(x));
            for (size_type i = mid; i < end; ++i)
            {
                double const v = p_.surfaces[sorted[i]].value;
                if (v - x > result)
                    break;
                result = min_of(result, this->surface_safety(sorted[i], pos));
            }
            for (size_type i = mid; i-- > beg;)
            {
                double const v = p_.surfaces[sorted[i]].value;
                if (x - v > result)
                    break;
                result = min_of(result, this->surface_safety(sorted[i], pos));
            }
        }
        // Cylinders: outward and inward from the point's radius, until the
        // FP32 bound above exceeds the minimum (it grows with |r - R|)
        size_type const cbeg = p_.sorted_offset[surf_czc];
        size_type const cend = p_.sorted_offset[surf_czc + 1];
        size_type const mid = key_lower_bound(key, cbeg, cend, rf);
        auto beyond = [&](size_type i) {
            float const best = static_cast<float>(result);
            float const margin = 1e-5f * (key[i] + rf + best) + 1e-6f;
            return std::fabs(rf - key[i]) - margin > best;
        };
        for (size_type i = mid; i < cend; ++i)
        {
            if (beyond(i))
                break;
            result = min_of(result, this->surface_safety(sorted[i], pos));
        }
        for (size_type i = mid; i-- > cbeg;)
        {
            if (beyond(i))
                break;
            result = min_of(result, this->surface_safety(sorted[i], pos));
        }
    }
#endif
    return result;
}

}  // namespace gbx
