"""Persistent-buffer sea-ice step for repeated time stepping on one GPU.

The drop-in routines (``veris_gb300.model.step``) allocate new output
tensors on every call, like the reference's functional kernels.  The engine
instead binds the C ABI once to fixed buffers and replays the same sequence
of launches every step, which makes the step capturable as one CUDA graph.

Precision modes:

* ``"f64"``: every kernel in float64 (the drop-in arithmetic);
* ``"f32"``: the EVP subcycles and the advection in float32 with float32
  accumulation; the dynamics preparation, ocean stress, clean-up, growth
  (with its solve4temp Newton solve and the heat/fresh-water/salt budgets)
  and all conservation sums stay float64, and the float64 state remains the
  master copy.

The step order is the reference setup's (veris/setup/seaice_global_4deg/
seaice_global_4deg.py:878-932), with all five EVP results stored back.
"""
import ctypes

import torch

from . import _abi
from ._abi import check
from .state import VerisState, require_device
from .variables import ABI_ORDER

# fields the float32 EVP and advection read that never change between steps
STATIC32 = ("maskInC", "maskInU", "maskInV", "iceMask", "iceMaskU", "iceMaskV",
            "k1AtC", "k2AtC", "k1AtZ", "k2AtZ", "Fu", "Fv", "fCori", "R_low",
            "dxC", "dyC", "dxG", "dyG", "dxU", "dyU", "dxV", "dyV",
            "recip_dxC", "recip_dyC", "recip_dxG", "recip_dyG",
            "recip_dxU", "recip_dyU", "recip_dxV", "recip_dyV",
            "rA", "rAu", "rAv", "rAz", "recip_rA", "recip_rAu", "recip_rAv", "recip_rAz")
# fields converted to float32 after the float64 dynamics preparation
DYNAMIC32 = ("uIce", "vIce", "sigma1", "sigma2", "sigma12",
             "SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "SeaIceStrength",
             "AreaW", "AreaS", "WindForcingX", "WindForcingY", "uOcean", "vOcean",
             "Area", "hIceMean", "hSnowMean")
EVP_OUT = ("uIce", "vIce", "sigma1", "sigma2", "sigma12")
GROWTH_OUT = ("hIceMean", "hSnowMean", "Area", "TSurf", "EmPmR", "forc_salt_surface_ice",
              "Qsw", "Qnet", "SeaIceLoad", "IcePenetSW", "recip_hIceMean")
# the prognostic fields the once-per-step non-finite check reads: a NaN in
# the dynamics reaches the velocities within the subcycles, one in the
# thermodynamics the thickness or the surface temperature
FINITE_CHECKED = ("uIce", "vIce", "hIceMean", "TSurf")
STATUS_NONFINITE = 2
FILLED_AFTER_GROWTH = ("hIceMean", "hSnowMean", "Area", "forc_salt_surface_ice", "Qnet")
# bit of veris_evp_fast_check: cell areas vary along both axes (the register
# walk needs them along j only)
V_AREA2D = 128
HELD_FORCING = ("Qnet", "Qsw")
# float64 conservation diagnostics recorded every step (budgets=True): area-
# weighted interior sums (veris/global_sum.py:1-4 is the hook the reference
# leaves for them; the budget quantities are those of veris/growth.py:296-383)
BUDGET_SLOTS = (
    "ice_volume_start", "snow_volume_start", "ice_area_start",            # sum rA*(h, hs, A) entering the step
    "ice_volume_advected", "snow_volume_advected", "ice_area_advected",   # after advection
    "ice_volume_cleaned", "snow_volume_cleaned",                          # after clean-up and ridging
    "ice_overshoot", "snow_overshoot",                                    # sum rA*(os_hIceMean, os_hSnowMean)
    "ice_volume_end", "snow_volume_end", "ice_area_end",                  # leaving the step
    "ocean_heat_loss", "fresh_water_flux", "salt_flux",                   # sum rA*(Qnet, EmPmR, forc_salt_surface_ice)
)
BUDGET_UNITS = ("m3", "m3", "m2", "m3", "m3", "m2", "m3", "m3", "m3", "m3", "m3", "m3", "m2", "W", "kg/s", "kg/s")
BUDGET_RING = 4096


class SeaIceStep:
    def __init__(self, state: VerisState, precision="f64", n_subcycles=None, evp="auto", hold_forcing=False,
                 f32_kernel="walk", walk_rows=0, walk_variant=0, check_finite=True, budgets=False):
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        if evp not in ("auto", "fast", "plain", "external"):
            raise ValueError("evp must be 'auto', 'fast', 'plain' or 'external'")
        if evp == "external" and precision != "f32":
            raise ValueError("an external EVP (the batched ensemble's) takes float32 velocities and stresses")
        if f32_kernel not in ("tma", "walk"):
            raise ValueError("f32_kernel must be 'tma' or 'walk'")
        self.state = state
        self.precision = precision
        self.f32_kernel = f32_kernel   # float32 fast form: register-walking warps or TMA-staged tiles
        self.walk_variant = int(walk_variant)
        self.lib = _abi.load()
        v = state.variables
        s = state.settings
        self.shape = tuple(v.iceMask.shape)
        self.device = v.iceMask.device
        self.walk_rows = int(walk_rows)   # 0: chosen by the library from the grid and the GPU
        NX, NY = self.shape
        self.n_sub = int(s.nEVPsteps if n_subcycles is None else n_subcycles)
        self.grid = _abi.VerisGrid(NX - 2 * s.olx, NY - 2 * s.oly, s.olx, s.oly, NY)
        self.params = _abi.params_from_settings(s)
        self.cells = (NX - 2 * s.olx) * (NY - 2 * s.oly)
        for n in ABI_ORDER:
            if getattr(v, n, None) is None:
                setattr(v, n, torch.zeros(self.shape, dtype=torch.float64, device=self.device))
            setattr(v, n, require_device(getattr(v, n), n, torch.float64, self.shape))
        self.f64 = _abi.VerisFields(**{n: getattr(v, n).data_ptr() for n in ABI_ORDER})
        e = lambda dt=torch.float64: torch.empty(self.shape, dtype=dt, device=self.device)
        self.evp_out = [e() for _ in EVP_OUT]
        self.tmp = [e() for _ in range(2)]
        viol = 0 if evp == "external" else self._fast_violations()
        # cell areas varying along both axes: only the register walk cannot
        # take them (it holds them per column); the tile forms can
        self.area2d = bool(viol & V_AREA2D)
        self.fast_violations = viol & ~V_AREA2D
        if self.area2d and precision == "f32" and self.f32_kernel == "walk":
            if int(self.lib.veris_evp_fast_settings_check(ctypes.byref(self.params))):
                self.fast_violations |= V_AREA2D   # the TMA form cannot run these settings either
            else:
                self.f32_kernel = "tma"
        if evp == "fast" and self.fast_violations:
            raise ValueError(f"the fast EVP form does not cover this state (violations {self.fast_violations:#x})")
        self.evp_form = ("external" if evp == "external" else
                         "plain" if (evp == "plain" or self.fast_violations) else "fast")
        esize = 8 if precision == "f64" else 4
        wsb = (256 if self.evp_form == "external" else
               self.lib.veris_evp_fast_workspace_bytes(ctypes.byref(self.grid), esize) if self.evp_form == "fast"
               else self.lib.veris_evp_workspace_bytes(ctypes.byref(self.grid), esize))
        self.ws_evp = torch.empty(wsb, dtype=torch.uint8, device=self.device)
        self.ws_adv = torch.empty(self.lib.veris_advection_workspace_bytes(ctypes.byref(self.grid), 8),
                                  dtype=torch.uint8, device=self.device)
        if precision == "f32":
            self.v32 = {n: e(torch.float32) for n in STATIC32 + DYNAMIC32}
            self.evp_out32 = [e(torch.float32) for _ in EVP_OUT]
            self.adv_out32 = [e(torch.float32) for _ in range(3)]
            # the EVP reads the velocities it starts from; the advection reads
            # the new ones: two float32 tables differing only in uIce/vIce
            self.f32 = _abi.VerisFields()
            for n in ABI_ORDER:
                if n in self.v32:
                    setattr(self.f32, n, self.v32[n].data_ptr())
            self.f32_adv = _abi.VerisFields.from_buffer_copy(self.f32)
            self.f32_adv.uIce = self.evp_out32[0].data_ptr()
            self.f32_adv.vIce = self.evp_out32[1].data_ptr()
            for n in STATIC32:
                self._to32(getattr(v, n), self.v32[n])
        # Growth overwrites Qnet and Qsw with the ocean's budgets; a run
        # with fixed surface forcing restores them before every step
        self.forcing = ({n: getattr(v, n).clone() for n in HELD_FORCING} if hold_forcing else None)
        self.graph = None
        self.launches_per_step = None
        # sticky device status word: STATUS_NONFINITE once a step has left a
        # NaN or an infinity in one of FINITE_CHECKED (one launch per step)
        self.check_finite = bool(check_finite)
        self.status_dev = torch.zeros(1, dtype=torch.int32, device=self.device)
        # fast forms: a buffer of veris_evp_tape_bytes() that the next eager
        # step's EVP fills with its subcycle states
        self.evp_tape = None
        # conservation diagnostics: BUDGET_SLOTS of every step into a ring
        # of BUDGET_RING steps on the device (four sums calls per step)
        self.budgets = bool(budgets)
        if self.budgets:
            self.budget_ring = torch.zeros((BUDGET_RING, len(BUDGET_SLOTS)), dtype=torch.float64,
                                           device=self.device)
            self.budget_count = torch.zeros(1, dtype=torch.int32, device=self.device)
            self.budget_ws = torch.empty(self.lib.veris_budget_workspace_bytes(), dtype=torch.uint8,
                                         device=self.device)

    def set_settings(self, **kw):
        """Change scalar settings (e.g. pStar, airIceDrag) between steps;
        drops a captured graph, whose launches hold the old values."""
        for k, val in kw.items():
            setattr(self.state.settings, k, val)
        self.params = _abi.params_from_settings(self.state.settings)
        self.graph = None

    def _fast_violations(self):
        """Settings and state properties the fast EVP form does not cover (0: none).
        The float32 register-walking kernel also runs the adaptive EVP."""
        walk = self.precision == "f32" and self.f32_kernel == "walk"
        check_settings = (self.lib.veris_evp_walk_settings_check if walk else
                          self.lib.veris_evp_fast_settings_check)
        bits = int(check_settings(ctypes.byref(self.params)))
        flag = torch.zeros(1, dtype=torch.int32, device=self.device)
        check("evp_fast_check", self.lib.veris_evp_fast_check(*self._refs(self.f64), flag.data_ptr(),
                                                              self.stream))
        return bits | int(flag.item())

    # ------------------------------------------------------------ helpers
    @property
    def stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _refs(self, fields):
        return ctypes.byref(self.grid), ctypes.byref(self.params), ctypes.byref(fields)

    def _budget(self, first, names, weighted, advance=False):
        """Enqueue the float64 interior sums of ``names`` (times rA where
        ``weighted``) into slots first.. of this step's ring row."""
        v = self.state.variables
        n = len(names)
        fields = (ctypes.c_void_p * n)(*[getattr(v, k).data_ptr() for k in names])
        rA = v.rA.data_ptr()
        weights = (ctypes.c_void_p * n)(*[rA if w else None for w in weighted])
        check("budget_sums", self.lib.veris_budget_sums_f64(
            ctypes.byref(self.grid), fields, weights, n, first, self.budget_ring.data_ptr(), BUDGET_RING,
            self.budget_count.data_ptr(), 1 if advance else 0, self.budget_ws.data_ptr(), self.budget_ws.numel(),
            self.stream))
        return 2

    def budget_records(self):
        """{slot name: float64 numpy array over the recorded steps, oldest
        first} (synchronises; at most the last BUDGET_RING steps)."""
        if not self.budgets:
            raise RuntimeError("SeaIceStep was built without budgets")
        import numpy as np
        n = int(self.budget_count.item())
        ring = self.budget_ring.cpu().numpy()
        k = min(n, BUDGET_RING)
        rows = np.array([ring[(n - k + t) % BUDGET_RING] for t in range(k)]).reshape(k, len(BUDGET_SLOTS))
        return {name: rows[:, q] for q, name in enumerate(BUDGET_SLOTS)}

    def _to32(self, src, dst):
        check("convert", self.lib.veris_convert_f64_to_f32(src.data_ptr(), dst.data_ptr(), src.numel(),
                                                           self.stream))

    def _to64(self, src, dst):
        check("convert", self.lib.veris_convert_f32_to_f64(src.data_ptr(), dst.data_ptr(), src.numel(),
                                                           self.stream))

    # --------------------------------------------------------------- step
    def _enqueue(self, evp_events=None, marks=None, growth_chunks=1):
        """Enqueue one step on the current stream; returns the launch count.
        ``marks(name)`` is called between phases (for event timing);
        with ``growth_chunks`` > 1 Growth runs as that many launches over
        consecutive row blocks, each followed by ``marks("growth_rows",
        (row_begin, row_end))``."""
        mark = marks if marks is not None else (lambda name, rows=None: None)
        mark("start")
        n = self._enqueue_prep()
        mark("preparation")
        n += self._enqueue_evp(evp_events)
        mark("evp")
        return n + self._enqueue_post(mark, growth_chunks)

    def _enqueue_prep(self):
        """The step up to the EVP: held forcing, the starting budgets and the
        dynamics preparation (veris/setup/seaice_global_4deg/
        seaice_global_4deg.py:879-888); returns the launch count."""
        lib, v, st = self.lib, self.state.variables, self.stream
        r64 = self._refs(self.f64)
        n = 0
        if self.forcing is not None:
            for name, t in self.forcing.items():
                getattr(v, name).copy_(t)
        if self.budgets:
            n += self._budget(0, ("hIceMean", "hSnowMean", "Area"), (True,) * 3)
        check("SeaIceMass", lib.veris_sea_ice_mass_f64(*r64, v.SeaIceMassC.data_ptr(), v.SeaIceMassU.data_ptr(),
                                                       v.SeaIceMassV.data_ptr(), st))
        check("AreaWS", lib.veris_area_ws_f64(*r64, v.AreaW.data_ptr(), v.AreaS.data_ptr(), st))
        check("WindForcingXY", lib.veris_wind_forcing_xy_f64(*r64, v.WindForcingX.data_ptr(),
                                                             v.WindForcingY.data_ptr(), st))
        check("SeaIceStrength", lib.veris_sea_ice_strength_f64(*r64, v.SeaIceStrength.data_ptr(), st))
        return n + 4

    def _enqueue_evp(self, evp_events=None):
        """IceVelocities (veris/dynsolver.py:87-102): the EVP loop (or free
        drift) and the results into the float64 state; with an external EVP
        the caller has written the float32 results to ``evp_out32`` and this
        only converts them.  Returns the launch count."""
        lib, v, st = self.lib, self.state.variables, self.stream
        r64 = self._refs(self.f64)
        n = 0
        if evp_events:
            evp_events[0].record()
        ws = (self.ws_evp.data_ptr(), self.ws_evp.numel(), st)
        sett = self.state.settings
        if sett.useFreedrift and not sett.useEVP:
            # veris/dynsolver.py:93-97: free-drift velocities, stresses as they are
            check("freedrift_solver", lib.veris_freedrift_solver_f64(*r64, self.evp_out[0].data_ptr(),
                                                                      self.evp_out[1].data_ptr(), st))
            n += 1
            if evp_events:
                evp_events[1].record()
            v.uIce.copy_(self.evp_out[0])
            v.vIce.copy_(self.evp_out[1])
            if self.precision == "f32":
                for name in ("hIceMean", "hSnowMean", "Area"):
                    self._to32(getattr(v, name), self.v32[name])
                self._to32(v.uIce, self.evp_out32[0])
                self._to32(v.vIce, self.evp_out32[1])
                n += 5
        elif self.evp_form == "external":
            for name in ("hIceMean", "hSnowMean", "Area"):   # the float32 advection's inputs
                self._to32(getattr(v, name), self.v32[name])
            n += 3
            if evp_events:
                evp_events[1].record()
            for name, t in zip(EVP_OUT, self.evp_out32):
                self._to64(t, getattr(v, name))
            n += len(EVP_OUT)
        elif self.precision == "f64" and self.evp_tape is not None:
            # keep every subcycle's state (gradients of many steps); eager only
            tape = self.evp_tape
            check("evp_tape", lib.veris_evp_fast_tape_f64(*r64, self.n_sub, *[t.data_ptr() for t in self.evp_out],
                                                           tape.data_ptr(), tape.numel() * tape.element_size(),
                                                           *ws))
            n += self.n_sub + 1
            if evp_events:
                evp_events[1].record()
            for name, t in zip(EVP_OUT, self.evp_out):
                getattr(v, name).copy_(t)
        elif self.precision == "f64":
            fn = lib.veris_evp_fast_solver_f64 if self.evp_form == "fast" else lib.veris_evp_solver_f64
            check("evp_solver", fn(*r64, self.n_sub, *[t.data_ptr() for t in self.evp_out], *ws))
            n += self.n_sub + (1 if self.evp_form == "fast" else 0)
            if evp_events:
                evp_events[1].record()
            for name, t in zip(EVP_OUT, self.evp_out):
                getattr(v, name).copy_(t)
        else:
            conv = DYNAMIC32 if self.evp_form == "plain" else ("hIceMean", "hSnowMean", "Area")
            for name in conv:
                self._to32(getattr(v, name), self.v32[name])
            n += len(conv)
            outs = [t.data_ptr() for t in self.evp_out32]
            if self.evp_form == "fast" and self.evp_tape is not None:
                # float32 states of every subcycle (register-walking kernel); eager only
                tape = self.evp_tape
                check("evp_tape_f32", lib.veris_evp_fast_tape_f32(*r64, self.n_sub, *outs, tape.data_ptr(),
                                                                   tape.numel() * tape.element_size(), *ws))
                n += self.n_sub + 1
            elif self.evp_form == "fast" and self.f32_kernel == "walk":
                check("evp_walk_f32", lib.veris_evp_walk_solver_f32(*r64, self.n_sub, self.walk_rows,
                                                                         self.walk_variant, *outs, *ws))
                n += self.n_sub + 1
            elif self.evp_form == "fast":
                check("evp_fast_f32", lib.veris_evp_fast_solver_f32(*r64, self.n_sub, *outs, *ws))
                n += self.n_sub + 1
            else:
                check("evp_solver_f32", lib.veris_evp_solver_f32(*self._refs(self.f32), self.n_sub, *outs, *ws))
                n += self.n_sub
            if evp_events:
                evp_events[1].record()
            for name, t in zip(EVP_OUT, self.evp_out32):
                self._to64(t, getattr(v, name))
            n += len(EVP_OUT)
        return n

    def _enqueue_post(self, mark=None, growth_chunks=1):
        """The step after the EVP: ocean stress, advection, clean-up,
        ridging, Growth, the halo fills, the closing budgets and the
        non-finite check (seaice_global_4deg.py:894-932); returns the launch
        count."""
        lib, v, st = self.lib, self.state.variables, self.stream
        r64 = self._refs(self.f64)
        mark = mark if mark is not None else (lambda name, rows=None: None)
        n = 0
        check("OceanStressUV", lib.veris_ocean_stress_uv_f64(*r64, v.OceanStressU.data_ptr(),
                                                             v.OceanStressV.data_ptr(), st))
        n += 1
        mark("ocean_stress")
        if self.precision == "f64":
            # the last advection phase reads only its workspace: in place is safe
            check("Advection", lib.veris_advection_f64(*r64, v.hIceMean.data_ptr(), v.hSnowMean.data_ptr(),
                                                       v.Area.data_ptr(), self.ws_adv.data_ptr(),
                                                       self.ws_adv.numel(), st))
            n += 5
        else:
            check("Advection_f32", lib.veris_advection_f32(*self._refs(self.f32_adv),
                                                           *[t.data_ptr() for t in self.adv_out32],
                                                           self.ws_adv.data_ptr(), self.ws_adv.numel(), st))
            n += 5
            for name, t in zip(("hIceMean", "hSnowMean", "Area"), self.adv_out32):
                self._to64(t, getattr(v, name))
            n += 3
        if self.budgets:
            n += self._budget(3, ("hIceMean", "hSnowMean", "Area"), (True,) * 3)
        mark("advection")
        # pointwise routines run in place on the state
        check("clean_up_advection", lib.veris_clean_up_advection_f64(
            *r64, v.hIceMean.data_ptr(), v.hSnowMean.data_ptr(), v.Area.data_ptr(), v.TSurf.data_ptr(),
            v.os_hIceMean.data_ptr(), v.os_hSnowMean.data_ptr(), st))
        check("ridging", lib.veris_ridging_f64(*r64, v.Area.data_ptr(), st))
        if self.budgets:
            n += self._budget(6, ("hIceMean", "hSnowMean", "os_hIceMean", "os_hSnowMean"), (True,) * 4)
        mark("clean_up")
        outs = [getattr(v, k).data_ptr() for k in GROWTH_OUT]
        if growth_chunks <= 1:
            check("Growth", lib.veris_growth_f64(*r64, *outs, st))
        else:
            NX = self.shape[0]
            for k in range(growth_chunks):
                i0, i1 = NX * k // growth_chunks, NX * (k + 1) // growth_chunks
                check("Growth", lib.veris_growth_rows_f64(*r64, *outs, i0, i1, st))
                mark("growth_rows", (i0, i1))
        n += 3 + max(growth_chunks, 1) - 1
        mark("growth")
        for name in FILLED_AFTER_GROWTH:
            check("fill_overlap", lib.veris_fill_overlap_f64(ctypes.byref(self.grid), ctypes.byref(self.params),
                                                             getattr(v, name).data_ptr(), st))
        n += len(FILLED_AFTER_GROWTH)
        if self.budgets:
            n += self._budget(10, ("hIceMean", "hSnowMean", "Area", "Qnet", "EmPmR", "forc_salt_surface_ice"),
                              (True,) * 6, advance=True)
        mark("fill")
        if self.check_finite:
            ptrs = (ctypes.c_void_p * len(FINITE_CHECKED))(*[getattr(v, k).data_ptr() for k in FINITE_CHECKED])
            check("check_finite", lib.veris_check_finite_f64(ctypes.byref(self.grid), ptrs, len(FINITE_CHECKED),
                                                             STATUS_NONFINITE, self.status_dev.data_ptr(), st))
            n += 1
        return n

    def status(self):
        """The sticky status bits of the steps so far (synchronises)."""
        return int(self.status_dev.item())

    def clear_status(self):
        self.status_dev.zero_()

    def check(self, status=None):
        """Raise VerisError(VERIS_ERR_NAN) when a step left a NaN or an
        infinity in the prognostic fields (``status``: a word already read)."""
        if (self.status() if status is None else int(status)) & STATUS_NONFINITE:
            raise _abi.VerisError("SeaIceStep: " + "/".join(FINITE_CHECKED), _abi.VERIS_ERR_NAN)

    def step(self):
        """Run one step (replays the CUDA graph when one was captured)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launches_per_step = self._enqueue()

    def capture(self):
        """Capture one step as a CUDA graph (after one eager warm-up step)."""
        self.step()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.launches_per_step = self._enqueue()
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return g

    def timed_step(self):
        """One eager step with CUDA events around the EVP phase; returns the
        EVP milliseconds after synchronising."""
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        self.launches_per_step = self._enqueue(evp_events=ev)
        ev[1].synchronize()
        return ev[0].elapsed_time(ev[1])

    def phase_times(self):
        """One eager step with CUDA events between its phases; returns
        {phase: milliseconds} after synchronising."""
        evs = []

        def mark(name, rows=None):
            e = torch.cuda.Event(enable_timing=True)
            e.record()
            evs.append((name, e))

        self._enqueue(marks=mark)
        evs[-1][1].synchronize()
        return {evs[k][0]: evs[k - 1][1].elapsed_time(evs[k][1]) for k in range(1, len(evs))}
