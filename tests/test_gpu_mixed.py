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
