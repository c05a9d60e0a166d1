"""The registry binding (CPU): install() puts every launcher factory into a
registry laid out like ``commkit._cuda`` under the reference's names, and
uninstall() restores what was there."""

from __future__ import annotations

import types

from commkit_gb300 import _cuda, plugin


def test_install_and_uninstall():
    reg = types.ModuleType("fake_commkit_cuda")
    original = {"llr": object(), "ldpc_layered": object(), "other": object()}
    reg._KERNEL_FACTORIES = dict(original)
    plugin.install(reg)
    for name in ("llr", "llr_separable_maxlog", "llr_separable", "ldpc_layered"):
        assert reg._KERNEL_FACTORIES[name] is _cuda._KERNEL_FACTORIES[name]
    assert reg._KERNEL_FACTORIES["other"] is original["other"]
    plugin.uninstall(reg)
    assert reg._KERNEL_FACTORIES == original


def test_get_kernel_names():
    assert sorted(_cuda._KERNEL_FACTORIES) == ["ldpc_layered", "llr", "llr_separable", "llr_separable_maxlog"]
    try:
        _cuda.get_kernel("nope")
    except KeyError as e:
        assert "registered" in str(e)
    else:
        raise AssertionError("unknown names raise KeyError")
