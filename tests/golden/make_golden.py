"""Generate the golden fixtures by running the reference plugin itself.

The reference (team-ocean/veris) is pure Python over the Veros operator API.
Veros is not installed here, so ``veros_shim/`` supplies the few Veros entry
points the plugin imports (single-process NumPy semantics); the plugin's own
``veris/*.py`` files then run unchanged, in float64 NumPy.

Usage (in a container that holds the reference checkout):

    python tests/golden/make_golden.py --reference PATH [--forcing | --plugin]

(PATH: the reference checkout; or set VERIS_REFERENCE.)

It writes one ``<case>.npz`` per case next to this script:

* ``in.<var>``: the initial state;
* ``settings``: the settings as a JSON string;
* ``seq.<kk>.<routine>.<output>``: the outputs of every call of one or more
  sea-ice steps, in the order of the reference setup's step
  (veris/setup/seaice_global_4deg/seaice_global_4deg.py:878-932), with the
  five-value ``IceVelocities`` result unpacked in full and the stresses stored
  back into the state;
* ``forcing.npz`` (``--forcing``): free drift and the bulk formula, see
  ``run_forcing``;
* ``residuals.npz`` (``--residuals``): the reference's residual branch with
  the two names it leaves unbound patched as ``run_residuals`` describes;
* ``setup_callsite.json`` and ``plugin.npz`` (``--plugin``): the call
  sequence of the reference setup's sea-ice step as its source writes it
  (``record_callsite``), and the plugin's ``set_inits`` on a host-model grid
  (``run_set_inits``);
* ``sub.<routine>.<output>``: single calls of the inner routines
  (strain rates, viscosities, drag coefficients, stress divergence, fluxes,
  limiter, solve4temp, one EVP subcycle) on the state after the dynamics
  preparation of the first step.

The fixtures are the parity anchor for the oracle (tests/test_oracle_golden.py)
and for the GPU kernels (tests/test_gpu_parity.py).
"""
import argparse
import copy
import json
import os
import sys
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

CASES = {
    # the first workload verbatim: 90x40 at 4 deg, dt 3600 s, 120 subcycles, from rest
    "c1": dict(grid=dict(nx=90, ny=40, seed=0), config="c1_4deg", steps=2, overrides={}),
    # moving ice with stresses, basal drag on, turning angles on
    "moving": dict(grid=dict(nx=36, ny=20, seed=1, init_velocity=0.2, init_stress=3000.0,
                             ice_lat=30.0),
                   config="c1_4deg", steps=2,
                   overrides=dict(nEVPsteps=30, basalDragK2=15.0, airTurnAngle=20.0,
                                  waterTurnAngle=15.0, sinWat=float(np.sin(np.deg2rad(15.0))),
                                  cosWat=float(np.cos(np.deg2rad(15.0))))),
    # odd sizes, free-slip side drag, adaptive EVP, absolute wind, sea-ice load,
    # doubly periodic halo fill, ice everywhere
    "small_a": dict(grid=dict(nx=21, ny=13, seed=2, init_velocity=0.1, init_stress=1000.0,
                              ice_lat=0.0),
                    config="c1_4deg", steps=1, sea_ice_load=True,
                    overrides=dict(nEVPsteps=10, noSlip=False, useAdaptiveEVP=True,
                                   useRelativeWind=False, useRealFreshWaterFlux=True,
                                   veros_fill=False)),
    # second-order no-slip terms, non-periodic x, wet y halo, an all-land row,
    # tensile strength
    "small_b": dict(grid=dict(nx=21, ny=13, seed=3, init_velocity=0.1, init_stress=1000.0,
                              ice_lat=20.0, land_fraction=0.4, wet_y_halo=True,
                              land_rows=(5,)),
                    config="c1_4deg", steps=1,
                    overrides=dict(nEVPsteps=10, secondOrderBC=True, enable_cyclic_x=False,
                                   tensileStrFac=0.05)),
    # no ice anywhere
    "noice": dict(grid=dict(nx=16, ny=10, seed=4, ice_lat=90.0),
                  config="c1_4deg", steps=1, overrides=dict(nEVPsteps=5)),
}


def _import_reference(ref):
    sys.path[:0] = [os.path.join(HERE, "veros_shim"), ref, REPO]
    import veris.area_mass as area_mass
    import veris.dynsolver as dynsolver
    import veris.dynamics_routines as dyn
    import veris.averaging as averaging
    import veris.evp_solver as evp
    import veris.ocean_stress as ocean_stress
    import veris.advection as advection
    import veris.clean_up as clean_up
    import veris.growth as growth
    import veris.solve4temp as s4t
    import veris.fill_overlap as fo
    import veris.freedrift_solver as fd
    import veris.heat_flux_MITgcm as heat_flux
    import importlib
    set_inits = importlib.import_module("veris.set_inits")   # the package binds the name to the function
    return SimpleNamespace(fd=fd, heat_flux=heat_flux, set_inits=set_inits, area_mass=area_mass,
                           dynsolver=dynsolver, dyn=dyn,
                           averaging=averaging, evp=evp, ocean_stress=ocean_stress,
                           advection=advection, clean_up=clean_up, growth=growth,
                           s4t=s4t, fo=fo)


def _state(arrays, sett):
    return SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in arrays.items()}),
                           settings=sett)


def _record(out, key, names, values):
    if not isinstance(values, tuple):
        values = (values,)
    assert len(names) == len(values), (key, len(values))
    for n, val in zip(names, values):
        out[f"{key}.{n}"] = np.array(val, dtype=np.float64)
        yield n, val


def run_case(R, case):
    from veris_gb300.synthetic import make_state, config_settings

    arrays = make_state(**case["grid"])
    if case.get("sea_ice_load"):
        rng = np.random.default_rng(99)
        arrays["SeaIceLoad"] = 900.0 * rng.random(arrays["hIceMean"].shape)
    sett = config_settings(case["config"], **case["overrides"])
    out = {f"in.{k}": v.copy() for k, v in arrays.items()}
    out["settings"] = np.array(json.dumps(vars(sett), sort_keys=True))
    state = _state(arrays, sett)
    vs = state.variables
    seq = 0

    def call(name, names, fn):
        nonlocal seq
        vals = fn(state)
        key = f"seq.{seq:02d}.{name}"
        seq += 1
        for n, val in _record(out, key, names, vals):
            setattr(vs, n, np.array(val, dtype=np.float64).copy())

    for step in range(case["steps"]):
        call("SeaIceMass", ("SeaIceMassC", "SeaIceMassU", "SeaIceMassV"), R.area_mass.SeaIceMass)
        call("AreaWS", ("AreaW", "AreaS"), R.area_mass.AreaWS)
        call("WindForcingXY", ("WindForcingX", "WindForcingY"), R.dynsolver.WindForcingXY)
        call("SeaIceStrength", ("SeaIceStrength",), R.dyn.SeaIceStrength)
        if step == 0:
            _inner_routines(R, state, out)
        call("IceVelocities", ("uIce", "vIce", "sigma1", "sigma2", "sigma12"),
             R.dynsolver.IceVelocities)
        call("OceanStressUV", ("OceanStressU", "OceanStressV"), R.ocean_stress.OceanStressUV)
        if step == 0:
            _advection_routines(R, state, out)
        call("Advection", ("hIceMean", "hSnowMean", "Area"), R.advection.Advection)
        call("clean_up_advection",
             ("hIceMean", "hSnowMean", "Area", "TSurf", "os_hIceMean", "os_hSnowMean"),
             R.clean_up.clean_up_advection)
        call("ridging", ("Area",), R.clean_up.ridging)
        if step == 0:
            _thermo_routines(R, state, out)
        call("Growth", ("hIceMean", "hSnowMean", "Area", "TSurf", "EmPmR",
                        "forc_salt_surface_ice", "Qsw", "Qnet", "SeaIceLoad",
                        "IcePenetSW", "recip_hIceMean"), R.growth.Growth)
        for n in ("hIceMean", "hSnowMean", "Area", "forc_salt_surface_ice", "Qnet"):
            call("fill_overlap", (n,), lambda st, n=n: R.fo.fill_overlap(st, getattr(vs, n).copy()))
    return out


def _inner_routines(R, state, out):
    vs = state.variables
    rec = lambda key, names, vals: list(_record(out, "sub." + key, names, vals))
    u, v = vs.uIce.copy(), vs.vIce.copy()
    e11, e22, e12 = R.dyn.strainrates(state, u, v)
    rec("strainrates", ("e11", "e22", "e12"), (e11, e22, e12))
    zeta, eta, press = R.dyn.viscosities(state, e11, e22, e12)
    rec("viscosities", ("zeta", "eta", "press"), (zeta, eta, press))
    rec("c_point_to_z_point", ("zetaZ",), R.averaging.c_point_to_z_point(state, zeta))
    rec("ocean_drag_coeffs", ("cDrag",), R.dyn.ocean_drag_coeffs(state, u, v))
    rec("basal_drag_coeffs", ("cBot",), R.dyn.basal_drag_coeffs(state, u, v))
    rec("side_drag", ("SideDragU", "SideDragV"), R.dyn.side_drag(state, u, v))
    rec("stressdiv", ("stressDivX", "stressDivY"),
        R.dyn.stressdiv(state, vs.sigma1.copy(), vs.sigma2.copy(), vs.sigma12.copy()))
    rec("tauXY", ("tauX", "tauY"), R.dynsolver.tauXY(state))
    one = copy.copy(state.settings)
    one.nEVPsteps = 1
    st1 = SimpleNamespace(variables=vs, settings=one)
    rec("evp_1", ("uIce", "vIce", "sigma1", "sigma2", "sigma12"), R.evp.evp_solver(st1))


def _advection_routines(R, state, out):
    vs = state.variables
    sett = state.settings
    rec = lambda key, names, vals: list(_record(out, "sub." + key, names, vals))
    uTrans = vs.uIce * vs.dyG * vs.iceMaskU
    vTrans = vs.vIce * vs.dxG * vs.iceMaskV
    rec("calc_ZonalFlux", ("ZonalFlux",),
        R.advection.calc_ZonalFlux(state, vs.hIceMean.copy(), uTrans))
    rec("calc_MeridionalFlux", ("MeridionalFlux",),
        R.advection.calc_MeridionalFlux(state, vs.hIceMean.copy(), vTrans))
    rec("calc_Advection", ("field",), R.advection.calc_Advection(state, vs.Area.copy()))
    cr = np.linspace(-3.0, 4.0, 141)
    out["sub.limiter.Cr"] = cr
    rec("limiter", ("phi",), R.advection.limiter(cr))


def _thermo_routines(R, state, out):
    vs = state.variables
    sett = state.settings
    rec = lambda key, names, vals: list(_record(out, "sub." + key, names, vals))
    hI = np.maximum(vs.hIceMean * 1.3, 0.05) * (vs.hIceMean > 0)
    hS = vs.hSnowMean * 1.3
    TempFrz = sett.tempFrz + sett.dtempFrz_dS * vs.ocSalt + sett.celsius2K
    out["sub.solve4temp.in_hIceActual"] = hI
    out["sub.solve4temp.in_hSnowActual"] = hS
    rec("solve4temp", ("TSurfOut", "F_io_net", "F_ia_net", "IcePenetSW", "FWsublim"),
        R.s4t.solve4temp(state, hI, hS, vs.TSurf.copy(), TempFrz))


def run_forcing(R):
    """``forcing.npz``: the routines beside the step, on inputs that reach
    their branches.

    * ``fd.<case>.*``: ``freedrift_solver`` (veris/freedrift_solver.py:5-62)
      on the state after the dynamics preparation of a case, and once with the
      wind and ocean set to zero on part of the domain (rhsN = 0 there);
    * ``bulk.*``: ``bulkf_formula_lanl`` (veris/heat_flux_MITgcm.py:5-123) on
      seeded air/sea values spanning stable and unstable layers, calm and
      strong winds;
    * ``res.<case>.*``: nothing from the reference (its residual branch does
      not run); the tests restate it."""
    from veris_gb300.synthetic import make_state, config_settings
    out = {}
    for name in ("moving", "small_b"):
        case = CASES[name]
        arrays = make_state(**case["grid"])
        sett = config_settings(case["config"], **case["overrides"])
        state = _state(arrays, sett)
        vs = state.variables
        for fn, names in ((R.area_mass.SeaIceMass, ("SeaIceMassC", "SeaIceMassU", "SeaIceMassV")),
                          (R.area_mass.AreaWS, ("AreaW", "AreaS")),
                          (R.dynsolver.WindForcingXY, ("WindForcingX", "WindForcingY"))):
            for n, val in zip(names, fn(state)):
                setattr(vs, n, np.array(val, dtype=np.float64))
        if name == "small_b":
            calm = np.zeros_like(vs.hIceMean, dtype=bool)
            calm[:, : calm.shape[1] // 3] = True
            for n in ("WindForcingX", "WindForcingY", "uOcean", "vOcean"):
                setattr(vs, n, np.where(calm, 0.0, getattr(vs, n)))
        for n in ("WindForcingX", "WindForcingY", "uOcean", "vOcean", "hIceMean", "fCori",
                  "iceMaskU", "iceMaskV"):
            out[f"fd.{name}.in.{n}"] = np.array(getattr(vs, n), dtype=np.float64)
        out[f"fd.{name}.settings"] = np.array(json.dumps(vars(sett), sort_keys=True))
        list(_record(out, f"fd.{name}", ("uIce", "vIce"), R.fd.freedrift_solver(state)))

    rng = np.random.default_rng(7)
    shape = (40, 28)
    uw = rng.normal(0.0, 8.0, shape)
    vw = rng.normal(0.0, 8.0, shape)
    uw[:3] *= 0.05                       # calm rows: |u| below 1 m/s
    vw[:3] *= 0.05
    uw[3, :4] = 0.0
    vw[3, :4] = 0.0                      # no wind at all
    tsf = 271.0 + 30.0 * rng.random(shape)
    ta = tsf + rng.normal(0.0, 6.0, shape)          # both signs of air-sea difference
    qa = 0.02 * rng.random(shape)
    ocn = (rng.random(shape) > 0.2).astype(np.float64)
    sett = config_settings("c1_4deg")
    state = _state(dict(hIceMean=np.zeros(shape)), sett)
    for n, val in (("uw", uw), ("vw", vw), ("ta", ta), ("qa", qa), ("tsf", tsf), ("ocn_mask", ocn)):
        out[f"bulk.in.{n}"] = val
    out["bulk.settings"] = np.array(json.dumps(vars(sett), sort_keys=True))
    list(_record(out, "bulk", ("flwupa", "flha", "fsha", "df0dT", "ust", "vst", "evp", "ssq",
                               "dEvdT"),
                 R.heat_flux.bulkf_formula_lanl(state, uw, vw, ta, qa, tsf, ocn)))
    return out


SETUP = os.path.join("veris", "setup", "seaice_global_4deg", "seaice_global_4deg.py")


def _table_names(path):
    """The keyword names of the dict(...) table in a plugin module."""
    import ast
    for node in ast.walk(ast.parse(open(path).read())):
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and node.func.id == "dict":
            return [k.arg for k in node.keywords]
    return []


def record_callsite(ref):
    """The sea-ice step of the reference setup as a call sequence: every
    assignment in the setup's forcing kernel, from the SeaIceMass call to the
    last halo fill, whose value is a call of a routine the setup imports
    from the plugin; per call the routine, its module, its arguments
    (``state`` or a state variable) and the variables it assigns.  Derived
    from the setup's syntax tree; no code is executed."""
    import ast
    path = os.path.join(ref, SETUP)
    tree = ast.parse(open(path).read())
    imports = {}
    for node in tree.body:
        if isinstance(node, ast.ImportFrom) and node.module and node.module.startswith("veris."):
            for a in node.names:
                imports[a.asname or a.name] = node.module

    def veris_call(stmt):
        return (isinstance(stmt, ast.Assign) and isinstance(stmt.value, ast.Call)
                and isinstance(stmt.value.func, ast.Name) and stmt.value.func.id in imports)

    def name_of(expr):
        if isinstance(expr, ast.Name):
            return expr.id
        if isinstance(expr, ast.Attribute) and isinstance(expr.value, ast.Name) and expr.value.id == "vs":
            return "vs." + expr.attr
        raise ValueError(f"unexpected argument {ast.dump(expr)}")

    for fn in ast.walk(tree):
        if not isinstance(fn, ast.FunctionDef):
            continue
        stmts = [st for st in fn.body if veris_call(st)]
        first = [k for k, st in enumerate(stmts) if st.value.func.id == "SeaIceMass"]
        if not first:
            continue
        calls = []
        for st in stmts[first[0]:]:
            tgt = st.targets[0]
            elts = tgt.elts if isinstance(tgt, ast.Tuple) else [tgt]
            calls.append({"line": st.lineno, "func": st.value.func.id, "module": imports[st.value.func.id],
                          "args": [name_of(a) for a in st.value.args],
                          "targets": [name_of(e)[3:] for e in elts]})
        return {"source": SETUP.replace(os.sep, "/"), "function": fn.name,
                "lines": [calls[0]["line"], calls[-1]["line"]], "calls": calls,
                "plugin_settings": sorted(_table_names(os.path.join(ref, "veris", "settings.py"))),
                "plugin_variables": sorted(_table_names(os.path.join(ref, "veris", "variables.py")))}
    raise RuntimeError("no function of the setup calls SeaIceMass")


def run_set_inits(R):
    """``plugin.npz``: the reference's set_inits (veris/set_inits.py:6-59)
    on a seeded host-model grid (3-level masks, 1-D grid spacings, 2-D
    areas, depth and Coriolis)."""
    rng = np.random.default_rng(11)
    NX, NY, NZ = 30, 18, 3
    ins = {
        "maskT": (rng.random((NX, NY, NZ)) > 0.3).astype(np.float64),
        "maskU": (rng.random((NX, NY, NZ)) > 0.35).astype(np.float64),
        "maskV": (rng.random((NX, NY, NZ)) > 0.35).astype(np.float64),
        "ht": 4000.0 * rng.random((NX, NY)),
        "coriolis_t": 1.4e-4 * (rng.random((NX, NY)) - 0.5),
        "dxt": 1e5 * (1.0 + rng.random(NX)), "dyt": 1e5 * (1.0 + rng.random(NY)),
        "dxu": 1e5 * (1.0 + rng.random(NX)), "dyu": 1e5 * (1.0 + rng.random(NY)),
        "area_t": 1e10 * (1.0 + rng.random((NX, NY))), "area_u": 1e10 * (1.0 + rng.random((NX, NY))),
        "area_v": 1e10 * (1.0 + rng.random((NX, NY))),
    }
    state = SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in ins.items()}),
                            settings=SimpleNamespace())
    R.set_inits.set_inits(state)
    out = {f"in.{k}": v for k, v in ins.items()}
    for k, v in vars(state.variables).items():
        if k not in ins:
            out[f"out.{k}"] = np.array(v, dtype=np.float64)
    return out


RESIDUAL_CASES = ("moving", "small_a", "small_b")
RESIDUAL_SUBCYCLES = 8


def run_residuals(R):
    """``residuals.npz``: the reference's own residual branch
    (veris/evp_solver.py:51-56, 191-230) on the state before the first EVP
    call of three golden cases, 8 subcycles each.

    As shipped the branch cannot run: it reads ``sigma11``/``sigma22``,
    names nothing binds (its subcycle body computes ``sig11``/``sig22``).
    What it means, and what is patched in here, in memory only: the stress
    components 0.5 * (sigma1 +- sigma2) of the state at that point of the
    body (the incoming state at :54-55, the updated one at :194-195).  The
    patch rewrites those two names in the body's syntax tree; nothing else
    changes.  The loop's final carry (which evp_solver drops) is captured by
    wrapping the module's for_loop; its resSig and resU entries are the
    residuals."""
    import ast
    import inspect
    import textwrap
    sys.path.insert(0, REPO)
    from tests import golden_io as G
    mod = R.evp
    tree = ast.parse(textwrap.dedent(inspect.getsource(mod.evp_solver_body)))

    class StressComponents(ast.NodeTransformer):
        def visit_Name(self, node):
            if isinstance(node.ctx, ast.Load) and node.id in ("sigma11", "sigma22"):
                pm = ast.Add() if node.id == "sigma11" else ast.Sub()
                both = ast.BinOp(ast.Name("sigma1", ast.Load()), pm, ast.Name("sigma2", ast.Load()))
                return ast.copy_location(ast.BinOp(ast.Constant(0.5), ast.Mult(), both), node)
            return node

    tree = ast.fix_missing_locations(StressComponents().visit(tree))
    body_orig, loop_orig = mod.evp_solver_body, mod.for_loop
    exec(compile(tree, mod.__file__, "exec"), mod.__dict__)
    carry = {}

    def capture(lo, hi, body, arg):
        carry["last"] = loop_orig(lo, hi, body, arg)
        return carry["last"]

    mod.for_loop = capture
    out = {}
    try:
        for case in RESIDUAL_CASES:
            g = G.load(case)
            first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
            st = G.state_before(g, first_evp)
            st.settings.computeEvpResidual = True
            st.settings.nEVPsteps = RESIDUAL_SUBCYCLES
            fields = mod.evp_solver(st)
            for n, a in zip(("uIce", "vIce", "sigma1", "sigma2", "sigma12"), fields):
                out[f"res.{case}.{n}"] = np.array(a, dtype=np.float64)
            out[f"res.{case}.resSig"] = np.array(carry["last"][15], dtype=np.float64)
            out[f"res.{case}.resU"] = np.array(carry["last"][16], dtype=np.float64)
    finally:
        mod.evp_solver_body, mod.for_loop = body_orig, loop_orig
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("VERIS_REFERENCE"),
                    help="the reference checkout (default: $VERIS_REFERENCE)")
    ap.add_argument("--cases", nargs="*", default=list(CASES))
    ap.add_argument("--forcing", action="store_true", help="write forcing.npz only")
    ap.add_argument("--plugin", action="store_true", help="write setup_callsite.json and plugin.npz only")
    ap.add_argument("--residuals", action="store_true", help="write residuals.npz only")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give --reference PATH or set VERIS_REFERENCE")
    np.seterr(all="ignore")    # the reference's where() evaluates both branches
    R = _import_reference(args.reference)
    if args.residuals:
        out = run_residuals(R)
        path = os.path.join(HERE, "residuals.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {len(out)} arrays")
        return
    if args.plugin:
        site = record_callsite(args.reference)
        path = os.path.join(HERE, "setup_callsite.json")
        with open(path, "w") as f:
            json.dump(site, f, indent=1)
        print(f"{path}: {len(site['calls'])} calls, lines {site['lines']}")
        out = run_set_inits(R)
        path = os.path.join(HERE, "plugin.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {len(out)} arrays")
        return
    if args.forcing:
        out = run_forcing(R)
        path = os.path.join(HERE, "forcing.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {len(out)} arrays, {os.path.getsize(path) / 1e6:.2f} MB")
        return
    for name in args.cases:
        out = run_case(R, CASES[name])
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {len(out)} arrays, {os.path.getsize(path) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
