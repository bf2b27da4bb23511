"""Python driver of an emitted program library (the reference's main.cpp role).

A Formura user's driver includes the generated header, calls ``Formura_Init``,
writes the initial state into the global arrays between ``navi.lower_*`` and
``navi.upper_*``, and calls ``Formura_Forward`` in a loop
(examples/pearson-3d-main.cpp:160-245, examples/diffusion-main.cpp:7-16).
:class:`FormuraProgram` does the same through ctypes: the globals are exposed
as numpy arrays that alias the library's memory, and the navigator as a
ctypes structure laid out like the emitted header's.
"""
from __future__ import annotations

import ctypes
import itertools
from pathlib import Path
from typing import Dict, Optional, Union

import numpy as np

from . import backend
from ._lib import FormuraError, STATUS_NAMES, lib as _core_lib
from .backend import Program, _delta_name


_C_TYPES = {"double": (ctypes.c_double, np.float64), "float": (ctypes.c_float, np.float32),
            "int": (ctypes.c_int, np.int32), "bool": (ctypes.c_bool, np.bool_)}


def navigator_type(p: Program):
    fields = [("time_step", ctypes.c_int)]
    for a in p.axis_names:
        fields += [("lower_" + a, ctypes.c_int), ("upper_" + a, ctypes.c_int),
                   ("offset_" + a, ctypes.c_int)]
    fields += [("mpi_comm_storage_", ctypes.c_uint64), ("mpi_my_rank", ctypes.c_int)]
    for d in itertools.product((-1, 0, 1), repeat=p.dim):
        fields.append((_delta_name(d), ctypes.c_int))
    return type("Formura_Navigator_" + p.name, (ctypes.Structure,), {"_fields_": fields})


class FormuraProgram:
    """One loaded ``lib<name>.so``: Formura_Init / Formura_Forward and globals."""

    def __init__(self, program: Program, so_path: Path):
        _core_lib()  # the engine must load; there is no other path
        self.program = program
        self.path = Path(so_path)
        self.lib = ctypes.CDLL(str(self.path))
        L = self.lib
        nav_t = navigator_type(program)
        self.navi = nav_t.in_dll(L, "navi")
        self._nav_ptr = ctypes.pointer(self.navi)
        for name in ("Formura_Init",):
            getattr(L, name).argtypes = [ctypes.POINTER(nav_t), ctypes.c_int]
        for name in ("Formura_Forward",):
            getattr(L, name).argtypes = [ctypes.POINTER(nav_t)]
        L.Formura_Advance.argtypes = [ctypes.POINTER(nav_t), ctypes.c_int]
        L.Formura_Device_State.argtypes = [ctypes.c_int]
        L.Formura_Device_State.restype = ctypes.c_void_p
        L.Formura_Set_Stream.argtypes = [ctypes.c_void_p]
        L.Formura_Conserved_Totals.argtypes = [ctypes.POINTER(ctypes.c_double)]
        L.Formura_Last_Error.restype = ctypes.c_char_p
        L.Formura_Monitor_Begin.argtypes = [ctypes.c_int, ctypes.c_int]
        L.Formura_Monitor_Wait.argtypes = [ctypes.c_void_p]
        L.Formura_Write_Monitor.argtypes = [ctypes.c_char_p, ctypes.c_int]
        self._monitor_axis = None
        n = int(np.prod(program.shape))
        self.state: Dict[str, np.ndarray] = {}
        self.state_names = [s for s, _ in program.states()]
        for s, t in program.states():
            ctype, dtype = _C_TYPES[t]
            buf = (ctype * n).in_dll(L, s)
            self.state[s] = np.frombuffer(buf, dtype=dtype).reshape(program.shape)
        self.steps_per_forward = program.steps_per_forward

    # -- error handling -------------------------------------------------------
    def _check(self, st: int, where: str):
        if st != 0:
            msg = (self.lib.Formura_Last_Error() or b"").decode(errors="replace")
            raise FormuraError(st, where, msg)

    # -- the generated API ------------------------------------------------------
    def init(self, comm: int = 0):
        self._check(self.lib.Formura_Init(self._nav_ptr, comm), "Formura_Init")

    def forward(self):
        self._check(self.lib.Formura_Forward(self._nav_ptr), "Formura_Forward")

    # -- extensions ---------------------------------------------------------------
    def upload(self):
        self._check(self.lib.Formura_Upload(), "Formura_Upload")

    def advance(self, n_forward: int = 1):
        self._check(self.lib.Formura_Advance(self._nav_ptr, int(n_forward)), "Formura_Advance")

    def download(self):
        self._check(self.lib.Formura_Download(), "Formura_Download")

    def device_state(self, index: int) -> int:
        p = self.lib.Formura_Device_State(int(index))
        if not p:
            raise FormuraError(2, "Formura_Device_State",
                               (self.lib.Formura_Last_Error() or b"").decode())
        return int(p)

    def set_stream(self, stream_ptr: int):
        self._check(self.lib.Formura_Set_Stream(ctypes.c_void_p(stream_ptr)), "Formura_Set_Stream")

    def conserved_totals(self) -> np.ndarray:
        k = len(self.state_names)
        out = (ctypes.c_double * k)()
        self._check(self.lib.Formura_Conserved_Totals(out), "Formura_Conserved_Totals")
        return np.array(out[:], dtype=np.float64)

    def monitor_begin(self, axis: int, index: int):
        """Start copying plane `index` of axis `axis` of every state array from
        the device (asynchronous: the stepping may continue meanwhile)."""
        self._check(self.lib.Formura_Monitor_Begin(int(axis), int(index)), "Formura_Monitor_Begin")
        self._monitor_axis = int(axis)

    def monitor_wait(self) -> Dict[str, np.ndarray]:
        """The planes started by :meth:`monitor_begin`, per state array."""
        if self._monitor_axis is None:
            raise FormuraError(1, "monitor_wait", "no plane in flight")
        a = self._monitor_axis
        pshape = [n for k, n in enumerate(self.program.shape) if k != a] or [1]
        dtypes = [self.state[n].dtype for n in self.state_names]
        sizes = [int(np.prod(pshape)) * d.itemsize for d in dtypes]
        buf = np.empty(sum(sizes), dtype=np.uint8)
        self._check(self.lib.Formura_Monitor_Wait(buf.ctypes.data), "Formura_Monitor_Wait")
        self._monitor_axis = None
        out, off = {}, 0
        for n, d, nb in zip(self.state_names, dtypes, sizes):
            out[n] = buf[off:off + nb].view(d).reshape(pshape).copy()
            off += nb
        return out

    def write_monitor(self, directory, rank: int = 0):
        """Monitor files of the device state, as the reference drivers write
        them from the host globals (examples/pearson-3d-main.cpp:116-157)."""
        self._check(self.lib.Formura_Write_Monitor(str(directory).encode(), int(rank)),
                    "Formura_Write_Monitor")

    def host_pinned(self) -> int:
        """How many state arrays' host globals are page-locked (0 before the
        first device use)."""
        return int(self.lib.Formura_Host_Pinned())

    def finalize(self):
        self._check(self.lib.Formura_Finalize(), "Formura_Finalize")


_loaded: Dict[str, FormuraProgram] = {}


def load_program(program: Union[str, Program], outdir: Optional[Path] = None) -> FormuraProgram:
    """Emit + build (if stale) and load a program library.  A program name is
    looked up in :data:`formura_gb300.programs.PROGRAMS`."""
    if isinstance(program, str):
        from .programs import PROGRAMS

        program = PROGRAMS[program]
    so = backend.build_program(program, outdir=outdir)
    key = str(so)
    if key not in _loaded:
        _loaded[key] = FormuraProgram(program, so)
    return _loaded[key]


__all__ = ["FormuraProgram", "load_program", "navigator_type", "FormuraError", "STATUS_NAMES"]
