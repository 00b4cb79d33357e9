"""Mixed-precision build against the FP64 build (GB300).

The mixed-precision library computes the physics in FP32 and keeps FP64 for
positions, geometry distances, time, the field integrator's error control
and the energy-deposition tally; its random streams diverge from the FP64
build's after a few steps, so agreement is statistical. Both builds
transport the same c2-like primaries (Urban MSC, 1 T field, 0.1-10 GeV e-)
in independent batches; the test requires

* total deposited energy within 0.5% of the FP64 build's,
* per-layer deposition consistent with the FP64 build's: chi-square over the
  100 calorimeter volumes with p > 0.01, errors from the batch-to-batch
  scatter of both builds,
* the same number of track-steps within 2%.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NUM_BATCHES = 16
PRIMARIES_PER_BATCH = 500
TOTAL_RTOL = 5e-3
CHI2_PMIN = 0.01
STEPS_RTOL = 2e-2


def transport_batches(gb, precision):
    from celeritas_gb300.workloads import WORKLOADS, make_primaries

    wl = WORKLOADS["c2"]
    params = gb.Params(gb.physics_file("calo"), "calo", field_tesla=wl["field"],
                       msc=wl["msc"], track_order="reindex_both_action",
                       precision=precision)
    edep, steps = [], []
    for b in range(NUM_BATCHES):
        st = gb.Stepper(params, 1 << 18, seed=1000 + b)
        prim = make_primaries(wl, num=PRIMARIES_PER_BATCH, seed_offset=b)
        res = [st.step(prim)] + st.run(max_steps=20000, batch=64)
        assert not (res[-1].alive or res[-1].queued), "transport did not finish"
        edep.append(st.energy_deposition())
        steps.append(sum(r.active for r in res))
    return np.array(edep), np.array(steps), params.detector_labels()


@pytest.fixture(scope="module")
def results(built_lib):
    import celeritas_gb300 as gb
    from celeritas_gb300.build import build

    gb.load_library(built_lib)
    gb.load_library(build(precision="mixed"), precision="mixed")
    return {p: transport_batches(gb, p) for p in ("double", "mixed")}


def test_total_energy_within_half_percent(results):
    d = results["double"][0].sum(axis=1)
    m = results["mixed"][0].sum(axis=1)
    rel = abs(m.mean() - d.mean()) / d.mean()
    assert rel < TOTAL_RTOL, (m.mean(), d.mean(), rel)


def test_per_layer_chi_square(results):
    from scipy import stats

    d = results["double"][0]
    m = results["mixed"][0]
    n = len(d)
    mean_d, mean_m = d.mean(axis=0), m.mean(axis=0)
    var = d.var(axis=0, ddof=1) / n + m.var(axis=0, ddof=1) / n
    used = var > 0
    chi2 = float((((mean_m - mean_d) ** 2)[used] / var[used]).sum())
    dof = int(used.sum())
    p = stats.chi2.sf(chi2, dof)
    assert p > CHI2_PMIN, (chi2, dof, p)


def test_track_steps_agree(results):
    sd = results["double"][1].sum()
    sm = results["mixed"][1].sum()
    assert abs(sm - sd) / sd < STEPS_RTOL, (sm, sd)


# Silicon tracker shells of the CMS-like geometry: inner radius of layer k,
# 0.3 mm thick
def si_inner_radius(k):
    return 4.0 + k * (110.0 - 4.0) / 9


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_cms_tracks_stay_in_their_volumes(built_lib, precision):
    """Every live track logically inside a silicon shell lies within it.

    FP32 physics directions are unit vectors only to FP32 rounding; the
    geometry must receive them renormalized, or its crossing distances are off
    by ~1e-7 of the distance and a track can be placed across a 0.3 mm shell
    into the wrong volume (it then deposits silicon energy loss over
    centimetres of gap).
    """
    import celeritas_gb300 as gb
    from celeritas_gb300.build import build
    from celeritas_gb300.workloads import WORKLOADS, make_primaries

    gb.load_library(build(precision=precision), precision=precision)
    wl = WORKLOADS["c3"]
    params = gb.Params(gb.physics_file("cms"), "cms", field_tesla=wl["field"], msc=True,
                       track_order="reindex_both_action", precision=precision)
    det = params.detector_labels()
    inner = np.full(len(det) + 1, np.nan)
    for k in range(10):
        inner[det.index(f"si_{k}")] = si_inner_radius(k)
    st = gb.Stepper(params, 1 << 16, seed=3, use_graph=False)
    st.step(make_primaries(wl, num=100))
    checked = 0
    for _ in range(60):
        st.step()
        status = st.get_state("status", np.uint8)
        d = st.get_state("detector", np.uint32).astype(np.int64)
        d = np.where(d < len(det), d, len(det))
        x = st.get_state("pos_x", np.float64)
        y = st.get_state("pos_y", np.float64)
        r = np.hypot(x, y)
        lo = inner[d]
        sel = np.isfinite(lo) & (status == 2)
        checked += int(sel.sum())
        outside = sel & ((r < lo - 1e-6) | (r > lo + 0.03 + 1e-6))
        assert not outside.any(), (
            f"{int(outside.sum())} tracks outside their silicon shell, e.g. r = "
            f"{r[outside][:3]} in layers {[det[i] for i in d[outside][:3]]}")
    assert checked > 100


CMS_BATCHES = 12
CMS_EVENTS_PER_BATCH = 10
CMS_PRIMARIES_PER_EVENT = 20


def cms_batches(gb, precision):
    """Per-volume deposition of CMS-like batches (3.8 T, MSC; e-/gamma of
    1-10 GeV, |eta| < 1.5), the same primaries for both builds"""
    from celeritas_gb300.primaries import eta_beam

    params = gb.Params(gb.physics_file("cms"), "cms", field_tesla=(0.0, 0.0, 3.8), msc=True,
                       track_order="reindex_both_action", precision=precision,
                       reentrant_looping=True)
    out = []
    n = CMS_EVENTS_PER_BATCH * CMS_PRIMARIES_PER_EVENT
    for b in range(CMS_BATCHES):
        st = gb.Stepper(params, 1 << 18, seed=300 + b)
        prim = eta_beam(n, emin=1000.0, emax=10000.0, pdgs=(11, 22), seed=50 + b,
                        num_events=CMS_EVENTS_PER_BATCH)
        res = [st.step(prim)] + st.run(max_steps=20000, batch=64)
        assert not (res[-1].alive or res[-1].queued), "transport did not finish"
        out.append(st.energy_deposition())
    return np.array(out)


def test_cms_mixed_agrees_with_fp64(built_lib):
    """CMS-like batches, paired by their primaries: per-volume chi-square
    (each volume's mean difference over its standard error, as the tail
    probability of a Student t turned into a normal deviate) with p > 0.01,
    and the total within 0.5%."""
    from scipy import stats

    import celeritas_gb300 as gb
    from celeritas_gb300.build import build

    gb.load_library(built_lib)
    gb.load_library(build(precision="mixed"), precision="mixed")
    fp64 = cms_batches(gb, "double")
    mixed = cms_batches(gb, "mixed")
    d = mixed - fp64
    n = len(d)
    se = d.std(axis=0, ddof=1) / np.sqrt(n)
    used = se > 0
    t = d.mean(axis=0)[used] / se[used]
    z = stats.norm.isf(stats.t.sf(np.abs(t), n - 1))
    chi2 = float((z ** 2).sum())
    dof = int(used.sum())
    p = stats.chi2.sf(chi2, dof)
    assert p > CHI2_PMIN, (chi2, dof, p)
    rel = abs(mixed.sum() - fp64.sum()) / fp64.sum()
    assert rel < TOTAL_RTOL, rel
