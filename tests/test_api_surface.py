"""The drop-in surface: every public call of the reference on this path
exists here with the same parameters (names, positional or keyword-only,
defaults), as recorded from the reference in ``api_signatures.json``.
Parameters this package adds must be keyword-only with a default.  CPU
only."""

from __future__ import annotations

import inspect
import json

import pytest

import commkit_gb300 as ck
from tests.conftest import GOLDEN

REF = json.loads((GOLDEN / "api_signatures.json").read_text())

# Defaults that differ on purpose: this package has no CPU path, so a
# Monte-Carlo run defaults to the current CUDA device, not "cpu".
DIFFERENT_DEFAULTS = {("coding.error_rate_curve", "device")}


def _ours(key: str):
    obj = ck
    for part in key.split(".", 1)[1].split("."):
        obj = getattr(obj, part)
    return obj


@pytest.mark.parametrize("key", sorted(REF))
def test_signature_matches_reference(key):
    ours = {n: p for n, p in inspect.signature(_ours(key)).parameters.items() if n != "self"}
    ref_names = [name for name, _, _ in REF[key]]
    # The reference's parameters, in its order, with its kinds and defaults.
    assert [n for n in ours if n in ref_names] == ref_names, (key, list(ours))
    for name, kind, default in REF[key]:
        p = ours[name]
        assert p.kind.name == kind, (key, name, p.kind.name, kind)
        if (key, name) in DIFFERENT_DEFAULTS:
            continue
        got = None if p.default is inspect.Parameter.empty else repr(p.default)
        assert got == default, (key, name, got, default)
    # Extras: keyword-only, with a default.
    for name, p in ours.items():
        if name not in ref_names:
            assert p.kind is inspect.Parameter.KEYWORD_ONLY and p.default is not inspect.Parameter.empty, (key, name)
