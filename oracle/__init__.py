"""Oracle for the ETDRK pseudo-spectral stepping path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package.  The product package ``exponax_gb300``
never imports it and has no CPU fallback through it.
"""

from . import exponax_np  # noqa: F401
