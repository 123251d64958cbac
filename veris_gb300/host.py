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


class HostCoupledStep:
    """Runs a ``SeaIceStep`` on host arrays: upload, step, download."""

    def __init__(self, engine, inputs=HOST_INPUTS, outputs=HOST_OUTPUTS):
        self.engine = engine
        self.inputs = tuple(inputs)
        self.outputs = tuple(outputs)
        v = engine.state.variables
        self.h2d_bytes = sum(getattr(v, n).numel() * getattr(v, n).element_size() for n in self.inputs)
        self.d2h_bytes = sum(getattr(v, n).numel() * getattr(v, n).element_size() for n in self.outputs)

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
        v = self.engine.state.variables
        for n in self.inputs:
            getattr(v, n).copy_(h_in[n], non_blocking=True)
        self.engine.step()
        for n in self.outputs:
            h_out[n].copy_(getattr(v, n), non_blocking=True)
        torch.cuda.current_stream(self.engine.device).synchronize()
        return h_out
