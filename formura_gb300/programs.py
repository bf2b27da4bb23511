"""The Formura programs this engine ships, one per workload.

Each is the GB300 counterpart of a ``.fmr`` + ``.yaml`` pair; the .fmr sources
are under ``examples/`` and name the form they follow in the reference.
"""
from __future__ import annotations

from .backend import Program

# Gray-Scott constants of the 3D workload: Du*dt/dx^2 = 0.1 (< 1/6, stable in 3D).
GS3D_CONSTANTS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)

PROGRAMS = {
    # 2D diffusion, examples/diffusion-2d.fmr: 256^2 FP64, coefficient
    # Dt/Dx**2 * (1/2)^2 = 0.1 on the 5-point difference, 1000 steps per Forward.
    "diffusion_2d": Program(
        name="diffusion_2d", form="diff2d_f64", intra_node_shape=(256, 256),
        constants=dict(Dt=0.4, Dx=1.0), monitor_interval=1000,
        temporal_blocking_interval=1, mpi_grid_shape=(1, 1)),
    # 3D Gray-Scott, examples/gray-scott-3d.fmr: 256^3 FP64, 2000 steps per Forward.
    "gray_scott_3d": Program(
        name="gray_scott_3d", form="gs3d_f64", intra_node_shape=(256, 256, 256),
        constants=GS3D_CONSTANTS, monitor_interval=2000,
        temporal_blocking_interval=1, mpi_grid_shape=(1, 1, 1)),
    # The same program in binary32 with Kahan time accumulation, temporally
    # blocked (temporal_blocking_interval 8: M = 2000 is a multiple of 2*8; the
    # kernel runs its tuned on-chip depth per HBM pass).
    "gray_scott_3d_f32k": Program(
        name="gray_scott_3d_f32k", form="gs3d_f32k_tb", intra_node_shape=(256, 256, 256),
        constants=GS3D_CONSTANTS, monitor_interval=2000,
        temporal_blocking_interval=8, mpi_grid_shape=(1, 1, 1)),
}
