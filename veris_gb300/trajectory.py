"""Gradients through many sea-ice steps on one GPU.

``Trajectory`` runs n steps of the sea-ice step (the engine's fast EVP
form in float64, or the engine's float32 step; surface forcing held fixed: Qnet and Qsw are restored before every
step, since Growth overwrites them with the ocean's budgets) and propagates
adjoints back through them with the hand-written adjoint kernels of every
routine of the step:

    prep -> EVP -> ocean stress -> advection -> clean-up + ridging -> Growth -> fills

The state one step hands to the next is CARRIED (velocities, stresses, ice
thickness, snow, concentration, surface temperature).  Step states are kept as
snapshots under a binomial checkpointing schedule: with s snapshot slots the
first split of every step range is the one that minimises the total number of
recomputed steps (a dynamic programme over (steps, slots)); with s >= n - 1
every step state is kept and nothing is recomputed.

Inside a step the adjoint recomputes the cheap routines (preparation,
advection, clean-up) from the step's start state; the new velocities come
from the next step's state (they are stored back unchanged), and the EVP
adjoint checkpoints its own subcycles.

``sea_ice_trajectory`` wraps this as a ``torch.autograd.Function`` with
gradients with respect to the initial hIceMean and Area and the coefficients
pStar, airIceDrag, airIceDrag_south, waterIceDrag and waterIceDrag_south.
"""
import ctypes

import torch

from ._abi import VerisFields, check
from .adjoint import EVP_STATE, EVP_FIELDS, ICE, PREP_OUT
from .engine import SeaIceStep

CARRIED = EVP_STATE + ICE
COEFFS = ("pStar", "airIceDrag", "airIceDrag_south", "waterIceDrag", "waterIceDrag_south")


def binomial_schedule(n, s):
    """Optimal first splits for reversing n steps with s snapshot slots.

    cost[k][t]: fewest step advances that reverse k steps starting from a held
    state with t free slots; split[k][t]: the number of steps to advance
    before storing the next snapshot.  cost[k][0] = k (k - 1) / 2 (recompute
    from the held state for every step) and
    cost[k][t] = min over m of m + cost[k - m][t - 1] + cost[m][t].
    """
    s = max(0, min(s, n - 1))
    cost = [[0] * (s + 1) for _ in range(n + 1)]
    split = [[1] * (s + 1) for _ in range(n + 1)]
    for k in range(2, n + 1):
        cost[k][0] = k * (k - 1) // 2
        for t in range(1, s + 1):
            if t >= k - 1:
                cost[k][t], split[k][t] = k - 1, 1
                continue
            best, bm = None, 1
            for m in range(1, k):
                c = m + cost[k - m][t - 1] + cost[m][t]
                if best is None or c < best:
                    best, bm = c, m
            cost[k][t], split[k][t] = best, bm
    return cost, split


def interior_mask(shape, olx=2, oly=2, device="cuda"):
    m = torch.zeros(shape, dtype=torch.float64, device=device)
    m[olx:shape[0] - olx, oly:shape[1] - oly] = 1.0
    return m


def tape_mode(tape, f32, every_step_snapshotted, n_steps, tape_bytes, taped_ws, free, fraction):
    """The EVP tape policy of a trajectory: True (every step's tape written
    during the forward), "step" (float32: one step's tape written during the
    reverse) or False (the EVP adjoint recomputes its subcycles).  ``tape``
    "auto" takes the first that fits in ``fraction`` of ``free`` bytes; an
    explicit choice is checked."""
    if tape == "auto":
        if every_step_snapshotted and (n_steps + 1) * tape_bytes <= fraction * free:
            return True
        if f32 and tape_bytes + taped_ws <= fraction * free:
            return "step"
        return False
    if tape == "step":
        if not f32:
            raise ValueError("tape='step' is a float32 form (the float64 adjoint's one-segment recompute "
                             "already runs the forward's own kernel)")
        return "step"
    if tape and not every_step_snapshotted:
        raise ValueError("taping needs every step snapshotted (snapshots=None)")
    return bool(tape)


class Trajectory:
    """n float64 steps from the state's current values and their adjoint."""

    def __init__(self, state, n_steps, n_subcycles=None, snapshots=None, evp_checkpoint_every=None, tape="auto",
                 tape_memory_fraction=0.6, precision="f64"):
        """``snapshots``: step snapshot slots (None: every step).  ``tape``:
        keep every EVP subcycle state of every step during the forward, so
        the adjoint recomputes no subcycle ("auto": when every step is
        snapshotted and the tapes fit in ``tape_memory_fraction`` of the free
        device memory).  ``tape="step"`` (float32 only): the reverse sweep
        writes the tape of one step at a time with the float32 register
        walk, just before that step's EVP adjoint, instead of the adjoint
        recomputing the subcycles in the shared-memory float32 form (3.7x
        slower per subcycle on 3600 x 1800); "auto" takes it for float32
        when the tapes of all steps do not fit and one does.  ``precision`` "f32": the forward is the engine's
        float32 step (float32 EVP and advection, float64 thermodynamics) and
        the EVP adjoint runs in float32; the other adjoints stay float64.
        ``evp_checkpoint_every``: without tapes, the EVP adjoint of a step
        recomputes its subcycles from checkpoints this many subcycles apart
        (0: one segment, every subcycle state of the step stored, the
        subcycles recomputed once; None: one segment when its store fits in
        ``tape_memory_fraction`` of the free device memory, else the spacing
        with the smallest workspace, about sqrt(subcycles))."""
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        self.precision = precision
        if state.settings.useRealFreshWaterFlux:
            raise ValueError("the step adjoint covers useRealFreshWaterFlux = False only")
        self.state = state
        self.n = int(n_steps)
        if self.n < 1:
            raise ValueError("n_steps must be >= 1")
        self.eng = SeaIceStep(state, precision, n_subcycles, evp="fast", hold_forcing=True)
        if precision == "f32" and self.eng.area2d:
            raise ValueError("float32 trajectories tape the register walk, which needs cell areas varying "
                             "along j only; use precision='f64' for this grid")
        self.lib = self.eng.lib
        self.snaps = self.n - 1 if snapshots is None else max(0, min(int(snapshots), self.n - 1))
        self.K = 0 if evp_checkpoint_every is None else int(evp_checkpoint_every)
        self._auto_K = evp_checkpoint_every is None
        self.cost, self.split = binomial_schedule(self.n, self.snaps)
        sh, dev = self.eng.shape, self.eng.device
        e = lambda: torch.empty(sh, dtype=torch.float64, device=dev)
        # recomputed intermediates of one step
        self.uv_next = [e(), e()]
        self.adv = [e() for _ in range(3)]                 # after advection
        self.cln = [e() for _ in range(4)]                 # after clean-up + ridging
        self.os = [e(), e()]
        # adjoints: the carried state at the step's end and start, and scratch
        self.lam = {k: e() for k in CARRIED}
        self.lam_new = {k: e() for k in CARRIED}
        self.lg = [e() for _ in range(3)]
        self.lc = {k: e() for k in ICE}
        self.la = [e() for _ in range(3)]
        self.lf = {k: e() for k in EVP_FIELDS if k not in ("hIceMean", "Area")}
        self.lscal = torch.zeros(len(COEFFS), dtype=torch.float64, device=dev)
        self.evp_scal = torch.zeros(2, dtype=torch.float64, device=dev)
        self.ocean_grad = {"uOcean": torch.zeros(sh, dtype=torch.float64, device=dev),
                           "vOcean": torch.zeros(sh, dtype=torch.float64, device=dev)}
        # field tables: the step's start state, the advection (new velocities),
        # the clean-up (advected ice), the ridging and the Growth (cleaned ice)
        base = self.eng.f64
        self.t_adv = VerisFields.from_buffer_copy(base)
        self.t_adv.uIce, self.t_adv.vIce = self.uv_next[0].data_ptr(), self.uv_next[1].data_ptr()
        self.t_cln = VerisFields.from_buffer_copy(base)
        self.t_cln.hIceMean, self.t_cln.hSnowMean, self.t_cln.Area = [t.data_ptr() for t in self.adv]
        self.t_rdg = VerisFields.from_buffer_copy(base)
        self.t_rdg.Area = self.cln[2].data_ptr()
        self.t_gro = VerisFields.from_buffer_copy(base)
        self.t_gro.hIceMean, self.t_gro.hSnowMean, self.t_gro.Area, self.t_gro.TSurf = \
            [t.data_ptr() for t in self.cln]
        self.t_gro.os_hIceMean, self.t_gro.os_hSnowMean = [t.data_ptr() for t in self.os]
        self.t_lf = VerisFields(**{k: t.data_ptr() for k, t in self.lf.items()})
        self.t_lprep = VerisFields(**{k: self.lf[k].data_ptr() for k in PREP_OUT})
        g = ctypes.byref(self.eng.grid)
        mk = lambda nbytes: torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
        self.ws_adv = mk(self.lib.veris_advection_adjoint_workspace_bytes(g))
        self.ws_prep = mk(self.lib.veris_prep_adjoint_workspace_bytes(g))
        f32 = precision == "f32"
        esize = 4 if f32 else 8
        tape_bytes = int(self.lib.veris_evp_tape_bytes(g, esize, self.eng.n_sub))
        taped_ws = int(self.lib.veris_evp_adjoint_taped_workspace_bytes_f32(g, self.eng.n_sub) if f32 else
                       self.lib.veris_evp_adjoint_taped_workspace_bytes(g, self.eng.n_sub))
        free = torch.cuda.mem_get_info(dev)[0] if tape == "auto" else 0
        tape = tape_mode(tape, f32, self.snaps == self.n - 1, self.n, tape_bytes, taped_ws, free,
                         tape_memory_fraction)
        self.tape_mode = "step" if tape == "step" else ("all" if tape else "off")
        tdt = torch.float32 if f32 else torch.float64
        # one tape, rewritten by every step's reverse
        self.step_tape = torch.empty(tape_bytes // esize, dtype=tdt, device=dev) if tape == "step" else None
        if tape == "step":
            tape = False
        self.tapes = ([torch.empty(tape_bytes // esize, dtype=tdt, device=dev) for _ in range(self.n)]
                      if tape else None)
        # the taped step is one CUDA graph writing this staging tape, copied
        # to the step's own tape after each replay (a graph holds fixed
        # addresses; the copy costs less than launching the step eagerly)
        self.tape_stage = torch.empty_like(self.tapes[0]) if tape else None
        self._tape_graph = None
        if tape or self.step_tape is not None:
            wsb = taped_ws
        else:
            if self._auto_K:
                self.K = self._fitting_checkpoint_spacing(g, esize, tape_memory_fraction)
            wsb = self.lib.veris_evp_adjoint_workspace_bytes(g, esize, self.eng.n_sub, self.K)
        self.ws_evp = mk(wsb)
        # float32 EVP adjoint: its state adjoints in float32
        self.l32 = ([torch.empty(sh, dtype=torch.float32, device=dev) for _ in range(10)] if f32 else None)
        self.snap = {}
        self._pool = []   # snapshot buffer sets no longer in use, reused before allocating
        self.stats = {"forward_steps": 0, "recomputed_steps": 0, "adjoint_steps": 0}
        self._graph_ok = False
        self.track_norms = False   # record |adjoint| after every step (a host sync per step)

    # ------------------------------------------------------------ state
    def _save(self):
        """A copy of the carried state, in a buffer set from the pool when
        one is free (no allocation inside a forward after the first)."""
        v = self.state.variables
        buf = self._pool.pop() if self._pool else [torch.empty_like(getattr(v, k)) for k in CARRIED]
        for t, k in zip(buf, CARRIED):
            t.copy_(getattr(v, k))
        return buf

    def _release(self, snap):
        if snap is not None:
            self._pool.append(snap)

    def _load(self, snap):
        v = self.state.variables
        for k, t in zip(CARRIED, snap):
            getattr(v, k).copy_(t)

    def _advance(self, m):
        for _ in range(m):
            self.eng.step()

    def set_coefficients(self, **kw):
        """Set any of COEFFS (plain floats) for the next forward/backward."""
        bad = set(kw) - set(COEFFS)
        if bad:
            raise KeyError(f"unknown coefficients {sorted(bad)}")
        self.eng.set_settings(**{k: float(x) for k, x in kw.items()})
        self._graph_ok = False

    def _ensure_graph(self):
        if not self._graph_ok:
            x = self._save()
            self.eng.capture()          # its eager warm-up step moves the state
            self._load(x)
            self._release(x)
            if self.tapes is not None:
                dev = self.eng.device
                g = torch.cuda.CUDAGraph()
                s = torch.cuda.Stream(dev)
                s.wait_stream(torch.cuda.current_stream(dev))
                self.eng.evp_tape = self.tape_stage
                try:
                    with torch.cuda.stream(s):
                        with torch.cuda.graph(g, stream=s):
                            self.eng.launches_per_step = self.eng._enqueue()
                finally:
                    self.eng.evp_tape = None
                torch.cuda.current_stream(dev).wait_stream(s)
                self._tape_graph = g
            self._graph_ok = True

    # ---------------------------------------------------------- forward
    def forward(self):
        """Run the n steps from the state's current carried values, storing
        the snapshots of the schedule's first descent.  Leaves the final
        state in the state's variables."""
        self._ensure_graph()
        for snap in self.snap.values():
            self._release(snap)
        self.snap = {0: self._save()}
        keep, pos, left, t = set(), 0, self.n, self.snaps
        while left > 1 and t > 0:
            m = self.split[left][t]
            pos += m
            keep.add(pos)
            left -= m
            t -= 1
        for k in range(1, self.n + 1):
            if self.tapes is not None:
                self._tape_graph.replay()
                self.tapes[k - 1].copy_(self.tape_stage)
            else:
                self.eng.step()
            if k in keep:
                self.snap[k] = self._save()
        v = self.state.variables
        self.uv_final = (v.uIce.clone(), v.vIce.clone())
        self.stats = {"forward_steps": self.n, "recomputed_steps": 0, "adjoint_steps": 0}

    # ---------------------------------------------------------- backward
    def backward(self, lam_final):
        """Adjoints at the start from ``lam_final`` ({name in CARRIED: tensor},
        missing names zero) at the end.  Returns ({name: adjoint of the
        initial value}, {coefficient: d/d coefficient}, {uOcean, vOcean:
        adjoint of the (constant) ocean velocities})."""
        if 0 not in self.snap:
            raise RuntimeError("backward() needs a forward() first")
        self._ensure_graph()
        for k in CARRIED:
            src = lam_final.get(k)
            if src is None:
                self.lam[k].zero_()
            else:
                self.lam[k].copy_(src)
        self.lscal.zero_()
        for t in self.ocean_grad.values():
            t.zero_()
        self.uv_next[0].copy_(self.uv_final[0])
        self.uv_next[1].copy_(self.uv_final[1])
        stack = [("rev", 0, self.n, self.snaps)]
        while stack:
            task = stack.pop()
            if task[0] == "free":
                self._release(self.snap.pop(task[1], None))
                continue
            _, lo, hi, t = task
            if hi - lo == 1:
                self._load(self.snap[lo])
                self._step_adjoint(lo)
                continue
            if t == 0:
                for k in range(hi - 1, lo - 1, -1):
                    self._load(self.snap[lo])
                    self._advance(k - lo)
                    self.stats["recomputed_steps"] += k - lo
                    self._step_adjoint(k)
                continue
            mid = lo + self.split[hi - lo][t]
            if mid not in self.snap:
                self._load(self.snap[lo])
                self._advance(mid - lo)
                self.stats["recomputed_steps"] += mid - lo
                self.snap[mid] = self._save()
            stack.append(("rev", lo, mid, t))
            stack.append(("free", mid))
            stack.append(("rev", mid, hi, t - 1))
        self._load(self.snap[0])
        grads = {k: self.lam[k].clone() for k in CARRIED}
        coeffs = {k: self.lscal[i].clone() for i, k in enumerate(COEFFS)}
        return grads, coeffs, {k: t.clone() for k, t in self.ocean_grad.items()}

    def _fitting_checkpoint_spacing(self, g, esize, fraction):
        """0 (one segment: the subcycles recomputed once) when that workspace
        fits in ``fraction`` of the free device memory; else the spacing
        with the smallest workspace (checkpoints plus one segment, about
        sqrt(subcycles) apart), which recomputes the subcycles twice."""
        n = self.eng.n_sub
        free = fraction * torch.cuda.mem_get_info(self.eng.device)[0]
        ws = lambda K: int(self.lib.veris_evp_adjoint_workspace_bytes(g, esize, n, K))
        if n < 2 or ws(0) <= free:
            return 0
        return min(range(1, n), key=ws)

    def _refs(self, table):
        return ctypes.byref(self.eng.grid), ctypes.byref(self.eng.params), ctypes.byref(table)

    def _step_adjoint(self, step):
        """self.lam (end of step k) -> self.lam (start of step k); the state's
        variables hold step k's start state, uv_next the velocities at its end."""
        lib, eng, v = self.lib, self.eng, self.state.variables
        st = eng.stream
        base = self._refs(eng.f64)
        for name, t in eng.forcing.items():
            getattr(v, name).copy_(t)
        # recompute: preparation (into the state), advection, clean-up, ridging
        check("SeaIceMass", lib.veris_sea_ice_mass_f64(*base, v.SeaIceMassC.data_ptr(), v.SeaIceMassU.data_ptr(),
                                                       v.SeaIceMassV.data_ptr(), st))
        check("AreaWS", lib.veris_area_ws_f64(*base, v.AreaW.data_ptr(), v.AreaS.data_ptr(), st))
        check("WindForcingXY", lib.veris_wind_forcing_xy_f64(*base, v.WindForcingX.data_ptr(),
                                                             v.WindForcingY.data_ptr(), st))
        check("SeaIceStrength", lib.veris_sea_ice_strength_f64(*base, v.SeaIceStrength.data_ptr(), st))
        check("Advection", lib.veris_advection_f64(*self._refs(self.t_adv), *[t.data_ptr() for t in self.adv],
                                                   eng.ws_adv.data_ptr(), eng.ws_adv.numel(), st))
        check("clean_up", lib.veris_clean_up_advection_f64(*self._refs(self.t_cln),
                                                           *[t.data_ptr() for t in self.cln],
                                                           *[t.data_ptr() for t in self.os], st))
        check("ridging", lib.veris_ridging_f64(*self._refs(self.t_rdg), self.cln[2].data_ptr(), st))

        lam, new = self.lam, self.lam_new
        # final fills of hIceMean, hSnowMean, Area
        for q, k in enumerate(ICE[:3]):
            check("fill_adjoint", lib.veris_fill_overlap_adjoint_f64(
                base[0], base[1], lam[k].data_ptr(), self.lg[q].data_ptr(), st))
        # Growth, at the cleaned state
        lc = [self.lc[k].data_ptr() for k in ICE]
        check("growth_adjoint", lib.veris_growth_adjoint_f64(
            *self._refs(self.t_gro), *[t.data_ptr() for t in self.lg], lam["TSurf"].data_ptr(), *lc, st))
        # clean-up + ridging, at the advected state; TSurf's adjoint is final
        check("cleanup_adjoint", lib.veris_cleanup_adjoint_f64(
            *self._refs(self.t_cln), *lc, *[t.data_ptr() for t in self.la], new["TSurf"].data_ptr(), st))
        # advection: into the start-state ice, and the new velocities' adjoints
        for k in ICE[:3]:
            new[k].zero_()
        check("advection_adjoint", lib.veris_advection_adjoint_f64(
            *self._refs(self.t_adv), *[t.data_ptr() for t in self.la], *[new[k].data_ptr() for k in ICE[:3]],
            lam["uIce"].data_ptr(), lam["vIce"].data_ptr(), self.ws_adv.data_ptr(), self.ws_adv.numel(), st))
        # EVP subcycles (adds hIceMean/Area through the basal drag into new)
        for t in self.lf.values():
            t.zero_()
        self.t_lf.hIceMean, self.t_lf.Area = new["hIceMean"].data_ptr(), new["Area"].data_ptr()
        if self.l32 is None:
            lo_ptrs = [lam[q].data_ptr() for q in EVP_STATE]
            li_ptrs = [new[q].data_ptr() for q in EVP_STATE]
            if self.tapes is not None:
                tape = self.tapes[step]
                check("evp_adjoint_taped", lib.veris_evp_adjoint_taped_f64(
                    *base, eng.n_sub, tape.data_ptr(), tape.numel() * 8, *lo_ptrs, *li_ptrs,
                    ctypes.byref(self.t_lf), self.evp_scal.data_ptr(), self.ws_evp.data_ptr(), self.ws_evp.numel(),
                    st))
            else:
                check("evp_adjoint", lib.veris_evp_adjoint_f64(
                    *base, eng.n_sub, self.K, *lo_ptrs, *li_ptrs, ctypes.byref(self.t_lf),
                    self.evp_scal.data_ptr(), self.ws_evp.data_ptr(), self.ws_evp.numel(), st))
        else:
            lo32, li32 = self.l32[:5], self.l32[5:]
            for q, name in enumerate(EVP_STATE):
                check("convert", lib.veris_convert_f64_to_f32(lam[name].data_ptr(), lo32[q].data_ptr(),
                                                              lo32[q].numel(), st))
            lo_ptrs = [t.data_ptr() for t in lo32]
            li_ptrs = [t.data_ptr() for t in li32]
            tape = self.tapes[step] if self.tapes is not None else self.step_tape
            if tape is self.step_tape and tape is not None:
                # this step's subcycles from its start state, as the forward ran them (the register
                # walk; the final state lands in the adjoint's input buffers, which it overwrites)
                check("evp_tape_f32", lib.veris_evp_fast_tape_f32(
                    *base, eng.n_sub, *li_ptrs, tape.data_ptr(), tape.numel() * 4, eng.ws_evp.data_ptr(),
                    eng.ws_evp.numel(), st))
            if tape is not None:
                check("evp_adjoint_taped_f32", lib.veris_evp_adjoint_taped_f32(
                    *base, eng.n_sub, tape.data_ptr(), tape.numel() * 4, *lo_ptrs, *li_ptrs,
                    ctypes.byref(self.t_lf), self.evp_scal.data_ptr(), self.ws_evp.data_ptr(), self.ws_evp.numel(),
                    st))
            else:
                check("evp_adjoint_f32", lib.veris_evp_adjoint_f32(
                    *base, eng.n_sub, self.K, *lo_ptrs, *li_ptrs, ctypes.byref(self.t_lf),
                    self.evp_scal.data_ptr(), self.ws_evp.data_ptr(), self.ws_evp.numel(), st))
            for q, name in enumerate(EVP_STATE):
                check("convert", lib.veris_convert_f32_to_f64(li32[q].data_ptr(), new[name].data_ptr(),
                                                              li32[q].numel(), st))
        self.lscal[3:5] += self.evp_scal
        self.ocean_grad["uOcean"] += self.lf["uOcean"]
        self.ocean_grad["vOcean"] += self.lf["vOcean"]
        # preparation: masses, areas, wind forcing, strength
        check("prep_adjoint", lib.veris_prep_adjoint_f64(
            *base, ctypes.byref(self.t_lprep), *[new[k].data_ptr() for k in ("hIceMean", "hSnowMean", "Area",
                                                                             "uIce", "vIce")],
            self.lscal.data_ptr(), self.ws_prep.data_ptr(), self.ws_prep.numel(), st))
        self.lam, self.lam_new = new, lam
        if self.track_norms:
            self.stats.setdefault("lam_norms", []).append(
                float(torch.sqrt(sum((new[q] * new[q]).sum() for q in CARRIED))))
        # this step's start velocities are the previous step's new ones
        self.uv_next[0].copy_(v.uIce)
        self.uv_next[1].copy_(v.vIce)
        self.stats["adjoint_steps"] += 1


def tracking_loss_adjoint(state, target, names=("uIce", "vIce", "Area")):
    """L = sum over the interior of (x - x*)^2 for x in ``names``; returns
    (L as a 0-d tensor, {name: dL/dx})."""
    v, s = state.variables, state.settings
    m = interior_mask(tuple(v.iceMask.shape), int(s.olx), int(s.oly), v.iceMask.device)
    L = torch.zeros((), dtype=torch.float64, device=v.iceMask.device)
    lam = {}
    for k in names:
        r = (getattr(v, k) - target[k]) * m
        L = L + (r * r).sum()
        lam[k] = 2.0 * r
    return L, lam


class _TrajectoryFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, hIceMean0, Area0, coeffs, traj):
        v = traj.state.variables
        traj.set_coefficients(**{k: float(coeffs[i]) for i, k in enumerate(COEFFS)})
        v.hIceMean.copy_(hIceMean0)
        v.Area.copy_(Area0)
        traj.forward()
        ctx.traj = traj
        ctx.coeffs_dtype = coeffs.dtype
        return v.uIce.clone(), v.vIce.clone(), v.Area.clone()

    @staticmethod
    def backward(ctx, gu, gv, gA):
        traj = ctx.traj
        lam = {k: g for k, g in zip(("uIce", "vIce", "Area"), (gu, gv, gA)) if g is not None}
        grads, coeffs, _ = traj.backward(lam)
        gc = torch.stack([coeffs[k] for k in COEFFS]).to(ctx.coeffs_dtype)
        return grads["hIceMean"], grads["Area"], gc, None


def sea_ice_trajectory(traj, hIceMean0, Area0, coeffs):
    """(uIce, vIce, Area) after ``traj.n`` steps from the state with hIceMean
    and Area replaced by ``hIceMean0``, ``Area0``; ``coeffs``: 1-D float64
    tensor of COEFFS.  Differentiable in all three (torch.autograd)."""
    return _TrajectoryFn.apply(hIceMean0, Area0, coeffs, traj)
