"""The constructor argument checks of the reference's MAC_CylinderFlow (solver/main.py:45-64),
in its order and with its messages, shared by every path of this library's MAC_CylinderFlow."""


def check_reference_arguments(boundary, transport, pressure_solver, time_scheme, ghost_pressure_extension,
                              ghost_velocity_interpolation):
    if boundary not in ('immersed', 'staircase', 'ghost_cell', 'cut_cell') or transport not in ('centered', 'upwind'):
        raise ValueError('Choose boundary=immersed/staircase/ghost_cell/cut_cell and transport=centered/upwind')
    if pressure_solver not in ('direct', 'iterative', 'cg_dct'):
        raise ValueError("pressure_solver must be direct, iterative or cg_dct")
    if pressure_solver == 'cg_dct' and boundary != 'cut_cell':
        raise ValueError("cg_dct is supported only for cut_cell")
    if boundary == 'immersed' and pressure_solver == 'iterative':
        raise NotImplementedError("pressure_solver='iterative' is currently supported for Cartesian/staircase/"
                                  "ghost-cell formulations. The immersed boundary projection uses the exact "
                                  "FFT/DCT Schur-complement direct solver.")
    if time_scheme not in ('legacy', 'ab2_cn'):
        raise ValueError('time_scheme must be legacy or ab2_cn')
    if time_scheme == 'ab2_cn' and (boundary not in ('cut_cell', 'ghost_cell') or transport != 'centered'):
        raise ValueError('ab2_cn requires cut_cell/ghost_cell and centered transport')
    if ghost_pressure_extension not in ('neumann', 'quadratic') or \
            ghost_velocity_interpolation not in ('bilinear', 'biquadratic'):
        raise ValueError('Unknown Ghost pressure extension or velocity interpolation')
    if (ghost_pressure_extension != 'neumann' or ghost_velocity_interpolation != 'bilinear') and \
            (boundary != 'ghost_cell' or time_scheme != 'ab2_cn'):
        raise ValueError('Ghost reconstruction options require Ghost AB2/CN')
