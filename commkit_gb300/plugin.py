"""Drop-in installation into the reference's kernel registry.

``install()`` puts this package's launcher factories into
``commkit._cuda._KERNEL_FACTORIES`` (``commkit/_cuda/__init__.py:69-81``)
under the reference's own names, so commkit's unchanged ``compute_llr`` and
``decode`` (``commkit/mapping/_demap.py:330,349``,
``commkit/coding/ldpc.py:566-581``) launch the sm_103a kernels on their CuPy
arrays: every constellation's demapper (``llr`` for non-separable ones,
the two separable ones) and both LDPC check rules (``ldpc_layered`` with
``sum_product`` False or True).  ``uninstall()`` restores the previous factories.
"""

from __future__ import annotations

from types import ModuleType
from typing import Any

from . import _cuda

NAMES = ("llr", "llr_separable_maxlog", "llr_separable", "ldpc_layered")

_saved: dict[str, Any] = {}


def install(cuda_module: ModuleType | None = None) -> ModuleType:
    """Register the launchers in ``commkit._cuda`` (or the given module)."""
    if cuda_module is None:
        import commkit._cuda as cuda_module  # type: ignore[no-redef]
    registry = cuda_module._KERNEL_FACTORIES
    for name in NAMES:
        if name not in _saved:
            _saved[name] = registry.get(name)
        registry[name] = _cuda._KERNEL_FACTORIES[name]
    return cuda_module


def uninstall(cuda_module: ModuleType | None = None) -> None:
    """Put back the factories ``install`` replaced."""
    if cuda_module is None:
        import commkit._cuda as cuda_module  # type: ignore[no-redef]
    registry = cuda_module._KERNEL_FACTORIES
    for name, factory in list(_saved.items()):
        if factory is None:
            registry.pop(name, None)
        else:
            registry[name] = factory
        del _saved[name]
