"""formura_gb300 — a GB300-native engine for the time-step loop of
Formura-generated stencil code.

The engine keeps the generated-code API of Formura's C back end
(src/Formura/MPICxx/Translate.hs:973-1139): a per-program header with
``struct Formura_Navigator``, the global state arrays, ``Formura_Init`` and
``Formura_Forward``.  The time steps run as hand-written sm_103a CUDA kernels
behind a thin C ABI (``include/formura_gb300.h``, ``libformura_gb300.so``).

Python entry points:
  * :func:`formura_gb300.runtime.load_program` — load (building if needed) an
    emitted program library and drive it through Formura_Init/Formura_Forward;
  * :mod:`formura_gb300.kernels` — the thin C ABI on torch device tensors;
  * :mod:`formura_gb300.inits` — seeded initial states of the shipped workloads.
"""
__version__ = "0.1.0"
