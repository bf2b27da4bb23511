"""Front end of the Formura language for the GB300 engine.

``parse`` (parser.py) -> ``build_om`` (om.py, the orthotope-machine graph of
``init`` and ``step``) -> ``manifest`` (mm.py, per-array cell programs grouped
into levels) -> ``emit_kernels`` (emit_cuda.py, one CUDA kernel per level).
:func:`compile_source` runs the first three; :func:`load_program` turns a
``.fmr`` file and its numerical-config ``.yaml`` into a backend Program whose
generated library keeps the reference's API (Formura_Init, Formura_Forward,
the navigator and the global state arrays).
"""
from __future__ import annotations

import functools
from pathlib import Path
from typing import Optional, Sequence

from . import config, mm, om, parser

__all__ = ["compile_source", "load_program", "parser", "om", "mm", "config"]


@functools.lru_cache(maxsize=64)
def compile_source(source: str, shape: Sequence[int]) -> mm.MMProgram:
    prog = parser.parse(source)
    omp = om.build_om(prog, list(shape))
    return mm.manifest(omp, list(shape))


def load_program(fmr_path, yaml_path=None, name: Optional[str] = None, **overrides):
    """A backend Program (form "fmr") from a .fmr file and its numerical
    config (``<name>.yaml`` beside it unless given); keyword arguments
    override config keys (intra_node_shape, mpi_grid_shape, monitor_interval,
    temporal_blocking_interval, and this engine's march_chunk, march_pair and
    tb_kernel)."""
    from ..backend import Program

    fmr_path = Path(fmr_path)
    yaml_path = Path(yaml_path) if yaml_path else fmr_path.with_suffix(".yaml")
    cfg = config.load(yaml_path) if yaml_path.exists() else {}
    cfg.update(overrides)
    if "intra_node_shape" not in cfg:
        raise ValueError("%s: intra_node_shape missing (no %s)" % (fmr_path, yaml_path))
    src = fmr_path.read_text(encoding="utf-8")
    pname = name or "fmr_" + fmr_path.stem.replace("-", "_")
    return Program(name=pname, form="fmr", intra_node_shape=list(cfg["intra_node_shape"]),
                   constants={}, monitor_interval=int(cfg.get("monitor_interval", 1)),
                   temporal_blocking_interval=int(cfg.get("temporal_blocking_interval", 1)),
                   mpi_grid_shape=cfg.get("mpi_grid_shape"), fmr_source=src,
                   march_chunk=int(cfg.get("march_chunk", 0)),
                   march_pair=int(cfg.get("march_pair", 0)),
                   tb_kernel=int(cfg.get("tb_kernel", 0)))
