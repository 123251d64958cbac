"""Stepping a host-resident state: the coupling a host-side ocean model uses.

The host model (Veros with its NumPy backend, say) owns the forcing and the
prognostic ice fields in host memory.  Every step the fields it owns are
copied to the device, the sea-ice step runs on the GPU, and the fields the
step produces are copied back, which is the sea-ice section of the
reference's setup (veris/setup/seaice_global_4deg/seaice_global_4deg.py:
840-979) with the arrays living on the host.  Grid and mask variables are
static: they are uploaded once with the state.
"""
import torch

# fields the host model provides each step: forcing and the prognostic ice state
HOST_INPUTS = ("uWind", "vWind", "wSpeed", "uOcean", "vOcean", "theta", "ocSalt", "Qnet", "Qsw",
               "SWdown", "LWdown", "ATemp", "aqh", "precip", "snowfall", "evap", "runoff",
               "surfPress", "ssh_an",
               "hIceMean", "hSnowMean", "Area", "TSurf", "uIce", "vIce", "sigma1", "sigma2", "sigma12")
# fields the step returns to the host model (the setup's KernelOutput set)
HOST_OUTPUTS = ("hIceMean", "hSnowMean", "Area", "TSurf", "uIce", "vIce", "sigma1", "sigma2", "sigma12",
                "EmPmR", "forc_salt_surface_ice", "Qsw", "Qnet", "SeaIceLoad", "IcePenetSW",
                "recip_hIceMean", "OceanStressU", "OceanStressV", "os_hIceMean", "os_hSnowMean")


# inputs only the clean-up (TSurf) and Growth (veris/growth.py,
# veris/solve4temp.py) read: their upload overlaps the dynamics
LATE_INPUTS = ("theta", "ocSalt", "Qnet", "Qsw", "SWdown", "LWdown", "ATemp", "aqh", "precip", "snowfall",
               "evap", "runoff", "wSpeed", "TSurf")
# outputs final once the ice velocities and the ocean stress are: their
# download overlaps advection and Growth
EARLY_OUTPUTS = ("uIce", "vIce", "sigma1", "sigma2", "sigma12", "OceanStressU", "OceanStressV")
# outputs final after the clean-up: their download overlaps Growth
MID_OUTPUTS = ("os_hIceMean", "os_hSnowMean")
# Growth runs as this many launches over row blocks; the rows of its outputs
# that one launch finished are downloaded while the next computes
GROWTH_CHUNKS = 4


def growth_row_plan(outputs, early_out, mid_out, NX, olx, veros_fill):
    """{output name: padded rows [lo, hi) final as soon as Growth has
    written them}.  Growth's outputs that the halo fill after Growth does not
    touch are final on all rows; the filled ones are final on the rows the
    x-halo fill leaves alone, unless the y halo is filled too (then columns
    of every row change and they wait for the fill)."""
    from .engine import FILLED_AFTER_GROWTH, GROWTH_OUT
    y_fill = not bool(veros_fill)
    plan = {}
    for n in outputs:
        if n not in GROWTH_OUT or n in early_out or n in mid_out:
            continue
        if n not in FILLED_AFTER_GROWTH:
            plan[n] = (0, NX)
        elif not y_fill:
            plan[n] = (int(olx), NX - int(olx))
    return plan


class HostCoupledStep:
    """Runs a ``SeaIceStep`` on host arrays: upload, step, download.

    With pinned host buffers the whole exchange is one CUDA graph per buffer
    set: the inputs the dynamics read are uploaded first, the fields only
    the clean-up and Growth read are uploaded on a second stream while the
    dynamics run, and
    on a third stream the velocities, stresses and ocean stress are
    downloaded while advection and Growth run, the overshoots of the
    clean-up while Growth runs, and Growth's outputs by row blocks while
    Growth computes the next block; the rows the halo fill rewrites follow
    the fill.  Other host buffers take the same order eagerly on one
    stream, Growth in one launch."""

    def __init__(self, engine, inputs=HOST_INPUTS, outputs=HOST_OUTPUTS, graph=True):
        self.engine = engine
        self.inputs = tuple(inputs)
        self.outputs = tuple(outputs)
        v = engine.state.variables
        self.h2d_bytes = sum(getattr(v, n).numel() * getattr(v, n).element_size() for n in self.inputs)
        self.d2h_bytes = sum(getattr(v, n).numel() * getattr(v, n).element_size() for n in self.outputs) + 4
        held = set(engine.forcing or ())   # restored on the main stream at the start of the step
        self.late = tuple(n for n in self.inputs if n in LATE_INPUTS and n not in held)
        self.early_out = tuple(n for n in self.outputs if n in EARLY_OUTPUTS)
        self.mid_out = tuple(n for n in self.outputs if n in MID_OUTPUTS)
        # Growth's outputs go out by rows while Growth runs
        s = engine.state.settings
        self.row_out = growth_row_plan(self.outputs, self.early_out, self.mid_out, engine.shape[0], s.olx,
                                       getattr(s, "veros_fill", True))
        self.use_graph = graph
        self.graphs = {}
        self._side_in = torch.cuda.Stream(engine.device)
        self._side_out = torch.cuda.Stream(engine.device)
        # the engine's status word comes back with the outputs: a step that
        # left non-finite values raises VerisError(VERIS_ERR_NAN)
        self._status_host = torch.zeros(1, dtype=torch.int32).pin_memory()

    def _enqueue(self, h_in, h_out, overlap):
        v = self.engine.state.variables
        main = torch.cuda.current_stream(self.engine.device)
        late = self.late if overlap else ()
        early_out = self.early_out if overlap else ()
        for n in self.inputs:
            if n not in late:
                getattr(v, n).copy_(h_in[n], non_blocking=True)
        if late:
            self._side_in.wait_stream(main)
            with torch.cuda.stream(self._side_in):
                for n in late:
                    getattr(v, n).copy_(h_in[n], non_blocking=True)

        mid_out = self.mid_out if overlap else ()
        row_out = self.row_out if overlap else {}
        done = {}   # rows of each row_out field already on their way

        def side(copies):
            self._side_out.wait_stream(main)
            with torch.cuda.stream(self._side_out):
                for dst, src in copies:
                    dst.copy_(src, non_blocking=True)

        def mark(name, rows=None):
            if name == "ocean_stress" and early_out:
                side([(h_out[n], getattr(v, n)) for n in early_out])
            elif name == "advection" and late:   # the clean-up comes next
                main.wait_stream(self._side_in)
            elif name == "clean_up" and mid_out:
                side([(h_out[n], getattr(v, n)) for n in mid_out])
            elif name == "growth_rows" and row_out:
                copies = []
                for n, (lo, hi) in row_out.items():
                    a, b = max(rows[0], lo), min(rows[1], hi)
                    if a < b:
                        copies.append((h_out[n][a:b], getattr(v, n)[a:b]))
                        done.setdefault(n, []).append((a, b))
                side(copies)

        self.engine.launches_per_step = self.engine._enqueue(
            marks=mark, growth_chunks=GROWTH_CHUNKS if row_out else 1)
        NX = self.engine.shape[0]
        for n in self.outputs:
            if n in early_out or n in mid_out:
                continue
            # the rows not sent yet (all of them for fields without early rows)
            sent = sorted(done.get(n, []))
            start = 0
            for a, b in sent + [(NX, NX)]:
                if start < a:
                    h_out[n][start:a].copy_(getattr(v, n)[start:a], non_blocking=True)
                start = max(start, b)
        self._status_host.copy_(self.engine.status_dev, non_blocking=True)
        if early_out or mid_out or row_out:
            main.wait_stream(self._side_out)

    def _checked(self, h_out):
        if self.engine.check_finite:
            self.engine.check(int(self._status_host[0]))
        return h_out

    def host_buffers(self):
        """Pinned host copies of the current device state (inputs, outputs)."""
        v = self.engine.state.variables
        h_in = {n: getattr(v, n).detach().cpu().pin_memory() for n in self.inputs}
        h_out = {n: torch.empty(getattr(v, n).shape, dtype=getattr(v, n).dtype).pin_memory()
                 for n in self.outputs}
        return h_in, h_out

    def step(self, h_in, h_out):
        """One step from host arrays ``h_in`` into host arrays ``h_out``;
        returns after the results are in host memory."""
        dev = self.engine.device
        pinned = all(h_in[n].is_pinned() for n in self.inputs) and all(h_out[n].is_pinned() for n in self.outputs)
        if not (self.use_graph and pinned):
            self._enqueue(h_in, h_out, overlap=pinned)
            torch.cuda.current_stream(dev).synchronize()
            return self._checked(h_out)
        key = (tuple(h_in[n].data_ptr() for n in self.inputs), tuple(h_out[n].data_ptr() for n in self.outputs))
        g = self.graphs.get(key)
        if g is None:
            self._enqueue(h_in, h_out, overlap=True)   # the step itself, eagerly, then the capture of the next
            torch.cuda.synchronize(dev)
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream(dev)
            s.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self._enqueue(h_in, h_out, overlap=True)
            torch.cuda.current_stream(dev).wait_stream(s)
            torch.cuda.synchronize(dev)
            self.graphs[key] = g
            return self._checked(h_out)
        g.replay()
        torch.cuda.current_stream(dev).synchronize()
        return self._checked(h_out)
