"""Drop-in for veris/evp_solver.py: the mEVP subcycling loop on the GPU."""
import torch

from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


# veris/evp_solver.py:18: print the residuals of every subcycle when they are computed
printEvpResidual = False
# (resU, resSig) of the last evp_solver call that computed residuals
last_residuals = None


@accepts_host_state
def evp_solver(state, n_subcycles=None):
    """veris/evp_solver.py:257-319 -> (uIce, vIce, sigma1, sigma2, sigma12).

    Runs ``settings.nEVPsteps`` subcycles (or ``n_subcycles``) from the
    state's velocities and stresses in float64, one tiled kernel per
    subcycle.  With ``settings.computeEvpResidual`` the residuals of every
    subcycle are computed as well (``evp_solver_residuals``), kept in the
    module's ``last_residuals`` and printed when its ``printEvpResidual`` is
    set, as in the reference (:227-234).
    """
    global last_residuals
    s = state.settings
    if s.computeEvpResidual:
        out = evp_solver_residuals(state, n_subcycles)
        last_residuals = (out[5], out[6])
        if printEvpResidual:
            for k, (ru, rs) in enumerate(zip(out[5].tolist(), out[6].tolist())):
                print("evp resU, resSigma: %i %e %e" % (k, ru, rs))
        return tuple(out[:5])
    n = int(s.nEVPsteps if n_subcycles is None else n_subcycles)
    c = Call(state)
    out = c.empty(5)
    ws, wsb = c.workspace(c.lib.veris_evp_workspace_bytes(c.refs()[0], 8))
    check("evp_solver", c.lib.veris_evp_solver_f64(*c.refs(), n, *[t.data_ptr() for t in out], ws, wsb,
                                                    c.stream))
    return tuple(out)


@accepts_host_state
def evp_solver_residuals(state, n_subcycles=None, precision="f64"):
    """The loop with the residual diagnostics of veris/evp_solver.py:193-234
    -> (uIce, vIce, sigma1, sigma2, sigma12, resU, resSig).

    resU[k], resSig[k] (float64, one per subcycle) are the interior sums
    that branch means to form after subcycle k: the squared changes of the
    velocities weighted by the masks and beta, and of the stress components
    sig11, sig22 = (sigma1 +- sigma2) / 2 and sigma12 weighted by alpha
    (adaptive or constant).  The reference's branch reads names it never
    binds (:54-56) and does not run; these are the sums it describes.
    ``precision`` "f32" runs the loop on a float32 state (sums still in
    float64)."""
    s = state.settings
    n = int(s.nEVPsteps if n_subcycles is None else n_subcycles)
    dt = torch.float32 if precision == "f32" else torch.float64
    c = Call(state, dtype=dt)
    out = c.empty(5)
    res = torch.zeros((2, max(n, 1)), dtype=torch.float64, device=c.device)
    ws, wsb = c.workspace(c.lib.veris_evp_residual_workspace_bytes(c.refs()[0], 4 if dt == torch.float32 else 8,
                                                                   n))
    fn = c.lib.veris_evp_residual_solver_f32 if dt == torch.float32 else c.lib.veris_evp_residual_solver_f64
    check("evp_solver_residuals", fn(*c.refs(), n, *[t.data_ptr() for t in out], res[0].data_ptr(),
                                     res[1].data_ptr(), ws, wsb, c.stream))
    return tuple(out) + (res[0, :n], res[1, :n])


def evp_solver_f32(state32, n_subcycles=None):
    """The same loop in float32 on a state whose variables are float32."""
    s = state32.settings
    n = int(s.nEVPsteps if n_subcycles is None else n_subcycles)
    c = Call(state32, dtype=torch.float32)
    out = c.empty(5)
    ws, wsb = c.workspace(c.lib.veris_evp_workspace_bytes(c.refs()[0], 4))
    check("evp_solver_f32", c.lib.veris_evp_solver_f32(*c.refs(), n, *[t.data_ptr() for t in out], ws,
                                                        wsb, c.stream))
    return tuple(out)


def evp_solver_fast(state, precision="f32", form="tma", n_subcycles=None, return_status=False, rows=16,
                    variant=0):
    """The fast forms of the loop on a float64 state: ``form`` "tma" (float32
    only: TMA-staged tiles), "walk" (float32 only: register-walking warps,
    ``rows`` output rows per walk) or "smem" (shared-memory tiles).  Results
    are in the arithmetic type.  Raises ``VerisError`` (status 7) for
    settings the fast forms do not cover, and ``ValueError`` for the walk on
    a state whose cell areas vary along both axes (it holds them per
    column)."""
    import ctypes
    s = state.settings
    n = int(s.nEVPsteps if n_subcycles is None else n_subcycles)
    c = Call(state)
    if precision == "f32" and form == "walk":
        flag = torch.zeros(1, dtype=torch.int32, device=c.device)
        check("evp_fast_check", c.lib.veris_evp_fast_check(*c.refs(), flag.data_ptr(), c.stream))
        if int(flag.item()) & 128:
            raise ValueError("the register walk needs cell areas varying along j only (V_AREA2D set)")
    dt = torch.float32 if precision == "f32" else torch.float64
    out = [torch.empty(c.shape, dtype=dt, device=c.device) for _ in range(5)]
    ws, wsb = c.workspace(c.lib.veris_evp_fast_workspace_bytes(c.refs()[0], 4 if precision == "f32" else 8))
    if precision == "f32" and form == "walk":
        check("evp_solver_walk", c.lib.veris_evp_walk_solver_f32(*c.refs(), n, int(rows), int(variant),
                                                                  *[t.data_ptr() for t in out], ws, wsb, c.stream))
    else:
        if precision == "f64":
            fn = c.lib.veris_evp_fast_solver_f64
        else:
            fn = c.lib.veris_evp_fast_solver_f32 if form == "tma" else c.lib.veris_evp_smem_solver_f32
        check("evp_solver_fast", fn(*c.refs(), n, *[t.data_ptr() for t in out], ws, wsb, c.stream))
    if return_status:
        st = ctypes.c_int32(-1)
        check("evp_fast_status", c.lib.veris_evp_fast_status(ws, ctypes.byref(st), c.stream))
        return tuple(out), st.value
    return tuple(out)
