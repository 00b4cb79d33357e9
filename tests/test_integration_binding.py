"""The reference-side binding of INTEGRATION.md, compiled and linked (no GPU).

INTEGRATION.md section 2 shows the adapter a maintainer adds to the
reference (GbxStepper, GbxStepAction). This test extracts its C++ blocks,
compiles them against the reference's own headers (with the oracle's
generated configuration headers) and this repository's C header, and links
them with the reference's host library (oracle/_ref) and the GB300 library,
so the documented binding stays true to both interfaces. It needs the
reference sources and is skipped where they are absent.
"""

import os
import re
import subprocess

import pytest

import oracle
from conftest import REPO

DRIVER = r"""
#include <memory>
// Never run: only makes every member of the binding emitted and linked
static void exercise(celeritas::GbxStepperInput const& inp,
                     std::shared_ptr<celeritas::ParticleParams const> particles,
                     celeritas::Span<celeritas::Primary const> primaries)
{
    celeritas::GbxStepper stepper(inp, particles);
    stepper.warm_up();
    celeritas::StepperResult r = stepper(primaries);
    r = stepper();
    stepper.kill_active();
    stepper.reseed(celeritas::UniqueEventId{0});
    celeritas::GbxStepAction action(celeritas::ActionId{0}, "pre-step",
                                    celeritas::StepActionOrder::pre, stepper.handle());
    (void)action.order();
    (void)r;
}

int main(int argc, char**)
{
    if (argc > 1000)
        exercise({}, nullptr, {});
    return 0;
}
"""


def binding_source() -> str:
    with open(os.path.join(REPO, "INTEGRATION.md")) as f:
        text = f.read()
    section = text[text.index("## 2. Reference-side binding"):text.index("## 3.")]
    blocks = re.findall(r"```cpp\n(.*?)```", section, re.S)
    assert len(blocks) == 2
    return "\n".join(blocks) + DRIVER


def test_binding_compiles_and_links(tmp_path):
    ref = oracle.reference_path()
    if not os.path.isdir(os.path.join(ref, "src", "celeritas")):
        pytest.skip("reference sources not present")
    if oracle.build_reference(ref) is None:
        pytest.skip("reference library not buildable here")
    from celeritas_gb300.build import build

    lib = build()
    src = tmp_path / "binding.cc"
    src.write_text(binding_source())
    exe = tmp_path / "binding"
    cmd = ["g++", "-std=c++17", "-O0", "-w",
           "-I", os.path.join(REPO, "include"),
           "-I", os.path.join(REPO, "oracle", "ref", "include"),
           "-I", os.path.join(ref, "src"),
           str(src), "-o", str(exe),
           os.path.join(REPO, "oracle", "_ref", "libceleritas_ref.a"),
           "-L", os.path.dirname(lib), "-l:" + os.path.basename(lib),
           "-Wl,-rpath," + os.path.dirname(lib), "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
