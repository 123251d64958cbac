"""Many independent sea-ice domains of uneven sizes, advanced together.

``Ensemble`` folds every member's float64 state into one device workspace
(float32 fast form: constants + ping-pong state per member) and advances all
members by one subcycle per launch of a persistent kernel that pulls tiles
from a global work queue.

With ``full_step=True`` one ensemble step is the whole sea-ice step of every
member (veris/setup/seaice_global_4deg/seaice_global_4deg.py:879-932):

    per member: dynamics preparation, fold of its EVP constants and state
    -> n_subcycles batched EVP launches over all members
    -> per member: velocities and stresses back into its float64 state, ocean
       stress, float32 advection, clean-up, ridging, float64 Growth, halo fills

with the per-member work spread over parallel branches (streams), captured
with the batched launches as one CUDA graph.  Without it (the dynamics-only
form) one step is

    refold (momentum constant from the current velocities; not on the first step)
    -> n_subcycles batched launches

and the members' thermodynamic state (ice strength, masses, areas, wind
forcing) is folded once at construction and held fixed.

``sequential_baseline`` runs the same members one after another through the
single-domain float32 solver (one call per member), the comparison the
batched form replaces.
"""
import ctypes

import torch

from . import _abi
from ._abi import VerisFields, VerisGrid, check
from .state import VerisState

EVP_STATE = ("uIce", "vIce", "sigma1", "sigma2", "sigma12")
# 0-3: shared-memory tiles (rows, columns); 4-6: register walks (rows, 28 columns)
SHAPES = {0: (32, 32), 1: (16, 32), 2: (32, 16), 3: (16, 16), 4: (8, 28), 5: (16, 28), 6: (32, 28), 7: (64, 28),
          8: (128, 28)}


def prepare_dynamics(lib, grid, params, fields, v, stream):
    """The step's dynamics preparation (SeaIceMass, AreaWS, WindForcingXY,
    SeaIceStrength) into the state's own variables."""
    r = (ctypes.byref(grid), ctypes.byref(params), ctypes.byref(fields))
    check("SeaIceMass", lib.veris_sea_ice_mass_f64(*r, v.SeaIceMassC.data_ptr(), v.SeaIceMassU.data_ptr(),
                                                   v.SeaIceMassV.data_ptr(), stream))
    check("AreaWS", lib.veris_area_ws_f64(*r, v.AreaW.data_ptr(), v.AreaS.data_ptr(), stream))
    check("WindForcingXY", lib.veris_wind_forcing_xy_f64(*r, v.WindForcingX.data_ptr(),
                                                         v.WindForcingY.data_ptr(), stream))
    check("SeaIceStrength", lib.veris_sea_ice_strength_f64(*r, v.SeaIceStrength.data_ptr(), stream))


def _grid_of(state):
    s = state.settings
    NX, NY = state.shape
    return VerisGrid(NX - 2 * s.olx, NY - 2 * s.oly, s.olx, s.oly, NY)


def _fields_of(state):
    from .state import Call
    c = Call(state)
    return c, c.fields


class Ensemble:
    """n_subcycles float32 fast-form subcycles per step for many domains."""

    def __init__(self, members, n_subcycles, shape=0, blocks_per_sm=0, prepare=True, full_step=False,
                 branches=16):
        """``members``: float64 VerisStates on one GPU sharing their settings
        (they may differ in size and fields).  With ``prepare`` the dynamics
        preparation runs on each member first.  ``full_step``: every step is
        the whole sea-ice step of every member, the per-member work on
        ``branches`` parallel streams."""
        if not members:
            raise ValueError("an ensemble needs at least one member")
        self.lib = _abi.load()
        self.n = len(members)
        self.n_sub = int(n_subcycles)
        self.settings = members[0].settings
        self.params = _abi.params_from_settings(self.settings)
        if int(self.lib.veris_evp_fast_settings_check(ctypes.byref(self.params))):
            raise ValueError("the ensemble's settings are outside the fast EVP form")
        self.device = members[0].variables.iceMask.device
        self.grids = (VerisGrid * self.n)(*[_grid_of(m) for m in members])
        self.shapes = [tuple(m.shape) for m in members]
        self.cells = [g.nx * g.ny for g in self.grids]
        self.shape = int(shape)
        self.blocks_per_sm = int(blocks_per_sm)
        wsb = self.lib.veris_batch_workspace_bytes(self.n, self.grids)
        if wsb == 0:
            raise ValueError("invalid member grids")
        self.ws = torch.empty(wsb, dtype=torch.uint8, device=self.device)
        check("batch_init", self.lib.veris_batch_init(self.n, self.grids, ctypes.byref(self.params),
                                                      self.ws.data_ptr(), wsb))
        stream = torch.cuda.current_stream(self.device).cuda_stream
        flag = torch.zeros(1, dtype=torch.int32, device=self.device)
        for m, st in enumerate(members):
            call, fields = _fields_of(st)
            if prepare:
                prepare_dynamics(self.lib, call.grid, self.params, fields, st.variables, stream)
            flag.zero_()
            check("evp_fast_check", self.lib.veris_evp_fast_check(
                ctypes.byref(call.grid), ctypes.byref(self.params), ctypes.byref(fields), flag.data_ptr(), stream))
            # bit 128 (cell areas along both axes) only changes how the
            # walks read the areas; the batch handles it per member
            if int(flag.item()) & ~128:
                raise ValueError(f"member {m} is outside the fast EVP form (violations {int(flag.item()):#x})")
            check("batch_prep_member", self.lib.veris_batch_prep_member_f32(
                self.n, self.grids, ctypes.byref(self.params), self.ws.data_ptr(), wsb, m, ctypes.byref(fields),
                stream))
        self.buf = 0
        self.first = True
        self.graphs = {}
        self.full_step = bool(full_step)
        if self.full_step:
            from .engine import SeaIceStep
            self.members = members
            # the members' own steps around the batched EVP (no EVP of their own)
            self.engines = [SeaIceStep(st, precision="f32", evp="external", check_finite=False)
                            for st in members]
            self.calls = [_fields_of(st)[0] for st in members]
            self.branches = [torch.cuda.Stream(self.device) for _ in range(max(1, int(branches)))]

    @property
    def stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    @property
    def total_tiles(self):
        return int(self.lib.veris_batch_tiles(self.n, self.grids, self.shape))

    def _enqueue(self, refold, buf, n_sub=None):
        check("batch_evp", self.lib.veris_batch_evp_f32(
            self.n, self.grids, ctypes.byref(self.params), self.ws.data_ptr(), self.ws.numel(),
            self.n_sub if n_sub is None else int(n_sub), buf, int(refold), self.shape, self.blocks_per_sm,
            self.stream))

    def _enqueue_full(self):
        """One whole sea-ice step of every member (see the module notes)."""
        main = torch.cuda.current_stream(self.device)
        wsb = self.ws.numel()
        nb = len(self.branches)
        for b in self.branches:
            b.wait_stream(main)
        for m, eng in enumerate(self.engines):
            with torch.cuda.stream(self.branches[m % nb]):
                eng._enqueue_prep()
                check("batch_prep_member", self.lib.veris_batch_prep_member_f32(
                    self.n, self.grids, ctypes.byref(self.params), self.ws.data_ptr(), wsb, m,
                    ctypes.byref(self.calls[m].fields), eng.stream))
        for b in self.branches:
            main.wait_stream(b)
        check("batch_evp", self.lib.veris_batch_evp_f32(
            self.n, self.grids, ctypes.byref(self.params), self.ws.data_ptr(), wsb, self.n_sub, 0, 0,
            self.shape, self.blocks_per_sm, main.cuda_stream))
        end = self.n_sub & 1
        for b in self.branches:
            b.wait_stream(main)
        for m, eng in enumerate(self.engines):
            with torch.cuda.stream(self.branches[m % nb]):
                check("batch_copy_state", self.lib.veris_batch_copy_state_f32(
                    self.n, self.grids, ctypes.byref(self.params), self.ws.data_ptr(), wsb, m, end,
                    *[t.data_ptr() for t in eng.evp_out32], eng.stream))
                eng._enqueue_evp()
                eng._enqueue_post()
        for b in self.branches:
            main.wait_stream(b)

    def step(self):
        """One ensemble step (a captured graph when ``capture`` ran)."""
        if self.full_step:
            g = self.graphs.get("full")
            if g is not None:
                g.replay()
            else:
                self._enqueue_full()
            self.buf = self.n_sub & 1
            return
        refold = not self.first
        key = (refold, self.buf)
        g = self.graphs.get(key)
        if g is not None:
            g.replay()
        else:
            self._enqueue(refold, self.buf)
        self.first = False
        self.buf ^= self.n_sub & 1

    def capture(self):
        """Capture the steady-state step (with refold) for each start buffer
        it can meet; the first step after construction still runs eagerly
        (run it before capturing: it also configures the kernels)."""
        if self.full_step:
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream(self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):   # records only: nothing runs
                    self._enqueue_full()
            torch.cuda.current_stream(self.device).wait_stream(s)
            self.graphs["full"] = g
            return
        bufs = (0, 1) if self.n_sub & 1 else (self.buf,)
        for b in bufs:
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream(self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):   # records only: nothing runs
                    self._enqueue(True, b)
            torch.cuda.current_stream(self.device).wait_stream(s)
            self.graphs[(True, b)] = g

    def set_launch(self, shape, blocks_per_sm):
        self.shape, self.blocks_per_sm = int(shape), int(blocks_per_sm)
        self.graphs = {}

    def state(self, m, dtype=torch.float32):
        """{name: tensor} of member m's current velocities and stresses (the
        batch's state after the last EVP)."""
        out = {k: torch.empty(self.shapes[m], dtype=torch.float32, device=self.device) for k in EVP_STATE}
        check("batch_copy_state", self.lib.veris_batch_copy_state_f32(
            self.n, self.grids, ctypes.byref(self.params), self.ws.data_ptr(), self.ws.numel(), m, self.buf,
            *[out[k].data_ptr() for k in EVP_STATE], self.stream))
        return {k: t.to(dtype) for k, t in out.items()}


def sequential_baseline(members, n_subcycles, outs=None, workspaces=None):
    """Each member through the single-domain float32 solver, one after the
    other (the members must be prepared).  Returns the per-member outputs."""
    lib = _abi.load()
    res = []
    for m, st in enumerate(members):
        call, fields = _fields_of(st)
        o = outs[m] if outs is not None else [torch.empty(st.shape, dtype=torch.float32, device=call.device)
                                              for _ in EVP_STATE]
        if workspaces is not None:
            ws = workspaces[m]
        else:
            ws = torch.empty(lib.veris_evp_fast_workspace_bytes(ctypes.byref(call.grid), 4), dtype=torch.uint8,
                             device=call.device)
        check("evp_fast_f32", lib.veris_evp_fast_solver_f32(
            ctypes.byref(call.grid), ctypes.byref(call.params), ctypes.byref(fields), int(n_subcycles),
            *[t.data_ptr() for t in o], ws.data_ptr(), ws.numel(), call.stream))
        res.append(o)
    return res
