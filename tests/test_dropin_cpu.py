"""The drop-in installer (diffsph_gb300.dropin) against the reference package itself.

The reference is imported from its source tree through tests/golden/ref_harness.py, from the
directory the DIFFSPH_REF_SRC environment variable names; without it these tests skip. Nothing is called on
a GPU: the checks are that every copy of every replaced name points at the drop-in after
``install``, that ``uninstall`` restores the reference's functions, and that each drop-in
keeps the reference function's parameter names.
"""
import importlib
import inspect
import os
import sys

import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def reference():
    sys.path.insert(0, GOLDEN)
    import ref_harness
    if not ref_harness.REF_SRC or not os.path.isdir(ref_harness.REF_SRC):
        pytest.skip("DIFFSPH_REF_SRC does not name the reference's src directory")
    return ref_harness.load_reference()


MODES = ["fused", "regions", "operators"]


@pytest.mark.parametrize("mode", MODES)
def test_install_replaces_every_copy_and_uninstall_restores(reference, mode):
    from diffsph_gb300 import dropin
    before = {(m, a): getattr(importlib.import_module(m), a) for m, a, _ in dropin.targets(mode)}
    replaced = dropin.install(mode)
    try:
        for m, a, new in dropin.targets(mode):
            assert getattr(importlib.import_module(m), a) is new, (m, a)
    finally:
        dropin.uninstall(replaced)
    for (m, a), f in before.items():
        assert getattr(importlib.import_module(m), a) is f, (m, a)


def test_dropins_keep_the_reference_signatures(reference):
    from diffsph_gb300 import dropin
    for mode in MODES:
        for m, a, new in dropin.targets(mode):
            ref = getattr(importlib.import_module(m), a)
            assert list(inspect.signature(new).parameters) == list(inspect.signature(ref).parameters), (m, a)


def test_unknown_mode_is_rejected():
    from diffsph_gb300 import dropin
    with pytest.raises(ValueError):
        dropin.targets("unknown")


@pytest.mark.parametrize("mode", MODES)
def test_every_by_name_copy_is_covered(reference, mode):
    """Every loaded reference module that holds (under the same name) a function the mode
    replaces is itself a target, so no call site of the step keeps the reference's version;
    the modules off the step (dropin.LEFT_ALONE, each with its reason) are skipped."""
    from diffsph_gb300 import dropin
    tg = dropin.targets(mode)
    covered = {(m, a) for m, a, _ in tg}
    originals = {a: getattr(importlib.import_module(m), a) for m, a, _ in tg}
    missed = []
    for name, mod in list(sys.modules.items()):
        if not name.startswith("diffSPH") or mod is None or name in dropin.LEFT_ALONE:
            continue
        for a, f in originals.items():
            if getattr(mod, a, None) is f and (name, a) not in covered:
                missed.append((name, a))
    assert not missed, missed
