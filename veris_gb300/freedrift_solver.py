"""Drop-in for veris/freedrift_solver.py: ice velocities without internal
stress, one warp-walking kernel."""
import torch

from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def freedrift_solver(state):
    """veris/freedrift_solver.py:5-62 -> (uIce, vIce), float64.

    Reads WindForcingX/Y, uOcean, vOcean, hIceMean, fCori, iceMaskU and
    iceMaskV of the state; every padded point of the result is written (the
    reference computes on the whole padded array)."""
    c = Call(state)
    u, v = c.empty(2)
    check("freedrift_solver", c.lib.veris_freedrift_solver_f64(*c.refs(), u.data_ptr(), v.data_ptr(),
                                                                c.stream))
    return u, v


def freedrift_solver_f32(state32):
    """The same on a state whose variables are float32."""
    c = Call(state32, dtype=torch.float32)
    u, v = c.empty(2)
    check("freedrift_solver_f32", c.lib.veris_freedrift_solver_f32(*c.refs(), u.data_ptr(), v.data_ptr(),
                                                                    c.stream))
    return u, v
