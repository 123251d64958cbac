"""CPU oracle of the sea-ice step: a float64 NumPy restatement.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline legs of ``bench.py`` may import this module, and only as the
checker (or as the timed CPU baseline), never as part of the product path.

Every function restates one routine of the reference plugin (team-ocean/veris)
and cites it.  Arrays are 2-D ``(nx + 2*olx, ny + 2*oly)`` float64, axis 0 = x.
Neighbour access wraps periodically over the PADDED array in both axes, as the
reference's ``roll`` does; ``shift(a, di, dj)[i, j] == a[i+di, j+dj]``.  The
arithmetic is written in the reference's order of operations, so on the same
inputs the results are bit-identical to the reference run through NumPy; the
golden fixtures in ``tests/golden`` (made by running the reference itself)
pin that.

``state`` is any object with ``.variables`` (attribute access to arrays) and
``.settings`` (attribute access to scalars).  Functions return new arrays and
never modify their inputs, except the halo fill, which, like the host model's,
fills its argument in place and returns it.
"""
import numpy as np


def shift(a, di, dj=0):
    """``a`` at (i+di, j+dj), periodic over the padded extent."""
    if di == 0 and dj == 0:
        return a
    return np.roll(a, (-di, -dj), axis=(0, 1))


def _sx(a, di):
    return np.roll(a, -di, axis=0)


def _sy(a, dj):
    return np.roll(a, -dj, axis=1)


# --------------------------------------------------------------------- halo

def fill_overlap(state, A):
    """veris/fill_overlap.py:6-18.

    ``veros_fill`` (the default) defers to the host model's single-process
    boundary copy: when the domain is cyclic in x, the last two columns get
    columns 2..3, then the first two get columns -4..-3; nothing happens
    otherwise.  Without it, a doubly periodic copy with the halo widths.
    """
    s = state.settings
    if s.veros_fill:
        if s.enable_cyclic_x:
            A[-2:, :] = A[2:4, :]
            A[:2, :] = A[-4:-2, :]
        return A
    ox, oy = s.olx, s.oly
    A[:ox, :] = A[-2 * ox:-ox, :]
    A[-ox:, :] = A[ox:2 * ox, :]
    A[:, :oy] = A[:, -2 * oy:-oy]
    A[:, -oy:] = A[:, oy:2 * oy]
    return A


def fill_overlap_uv(state, U, V):
    """veris/fill_overlap.py:21-23."""
    return fill_overlap(state, U), fill_overlap(state, V)


def global_sum(A):
    """veris/global_sum.py:1-4 (an identity on one process)."""
    return A


# ----------------------------------------------------------- step preparation

def AreaWS(state):
    """veris/area_mass.py:5-14: ice concentration at U and V points."""
    A = state.variables.Area
    return 0.5 * (A + _sx(A, -1)), 0.5 * (A + _sy(A, -1))


def SeaIceMass(state):
    """veris/area_mass.py:17-28: ice+snow mass at C, U and V points."""
    v, s = state.variables, state.settings
    mC = s.rhoIce * v.hIceMean + s.rhoSnow * v.hSnowMean
    return mC, 0.5 * (mC + _sx(mC, -1)), 0.5 * (mC + _sy(mC, -1))


def SeaIceStrength(state):
    """veris/dynamics_routines.py:5-18: P = P* h exp(-C*(1-A)), masked."""
    v, s = state.variables, state.settings
    return s.pStar * v.hIceMean * np.exp(-s.cStar * (1 - v.Area)) * v.iceMask


def tauXY(state):
    """veris/dynsolver.py:7-47: air-ice stress at U and V points."""
    v, s = state.variables, state.settings
    sinWin = np.sin(np.deg2rad(s.airTurnAngle))
    cosWin = np.cos(np.deg2rad(s.airTurnAngle))
    if s.useRelativeWind:
        urel = v.uWind - 0.5 * (v.uIce + _sx(v.uIce, 1))
        vrel = v.vWind - 0.5 * (v.vIce + _sy(v.vIce, 1))
    else:
        urel, vrel = v.uWind, v.vWind
    speed_sq = urel ** 2 + vrel ** 2
    with np.errstate(invalid="ignore"):
        speed = np.where(speed_sq < s.wSpeedMin ** 2, s.wSpeedMin, np.sqrt(speed_sq))
    cd = np.where(v.fCori < 0, s.airIceDrag_south, s.airIceDrag) * s.rhoAir * speed
    sgn = np.sign(v.fCori)
    tx = cd * (cosWin * urel - sgn * sinWin * vrel)
    ty = cd * (cosWin * vrel + sgn * sinWin * urel)
    return (0.5 * (tx + _sx(tx, -1)) * v.iceMaskU,
            0.5 * (ty + _sy(ty, -1)) * v.iceMaskV)


def WindForcingXY(state):
    """veris/dynsolver.py:50-84: wind stress times area plus surface tilt."""
    v, s = state.variables, state.settings
    tauX, tauY = tauXY(state)
    fx = tauX * v.AreaW
    fy = tauY * v.AreaS
    phi = s.gravity * v.ssh_an
    if s.useRealFreshWaterFlux:
        phi = phi + (v.surfPress + v.SeaIceLoad * s.gravity * s.seaIceLoadFac) * s.recip_rhoSea
    else:
        phi = phi + v.surfPress * s.recip_rhoSea
    fx = fx - v.SeaIceMassU * v.recip_dxC * (phi - _sx(phi, -1))
    fy = fy - v.SeaIceMassV * v.recip_dyC * (phi - _sy(phi, -1))
    return fx, fy


# ------------------------------------------------------------ EVP building blocks

def c_point_to_z_point(state, C, noSlip=True):
    """veris/averaging.py:4-19: wet-cell-normalised 4-point mean at Z points."""
    m = state.variables.iceMask
    n = m + _sx(m, -1)
    n = n + _sy(n, -1)
    with np.errstate(divide="ignore"):
        if noSlip:
            n = np.where(n > 0, 1.0 / n, 0.0)
        else:
            n = np.where(n == 4.0, 0.25, 0.0)
    z = C + _sx(C, -1)
    return n * (z + _sy(z, -1))


def strainrates(state, u, vv):
    """veris/dynamics_routines.py:143-217: e11, e22 at C, e12 at Z."""
    v, s = state.variables, state.settings
    u_e = _sx(u, 1)
    v_n = _sy(vv, 1)
    dudx = (u_e - u) * v.recip_dxU
    uave = (u_e + u) * 0.5
    dvdy = (v_n - vv) * v.recip_dyV
    vave = (v_n + vv) * 0.5
    e11 = (dudx + vave * v.k2AtC) * v.maskInC
    e22 = (dvdy + uave * v.k1AtC) * v.maskInC

    u_s = _sy(u, -1)
    v_w = _sx(vv, -1)
    dudy = (u - u_s) * v.recip_dyU
    uave = (u + u_s) * 0.5
    dvdx = (vv - v_w) * v.recip_dxV
    vave = (vv + v_w) * 0.5
    mz = v.iceMask * _sx(v.iceMask, -1)
    mz = mz * _sy(mz, -1)
    e12 = 0.5 * (dudy + dvdx - v.k1AtZ * vave - v.k2AtZ * uave) * mz
    if s.noSlip:
        hU = v.iceMaskU - _sy(v.iceMaskU, -1)
        hV = v.iceMaskV - _sx(v.iceMaskV, -1)
        e12 = e12 + (2.0 * uave * v.recip_dyU * hU + 2.0 * vave * v.recip_dxV * hV)
    if s.noSlip and s.secondOrderBC:
        mU, mV = v.iceMaskU, v.iceMaskV
        hU = (mU - _sx(mU, -1)) / 3.0
        hV = (mV - _sy(mV, -1)) / 3.0
        hU = hU * (_sx(mU, -2) * _sx(mU, -1) + _sx(mU, 1) * mU)
        hV = hV * (_sy(mV, -2) * _sy(mV, -1) + _sy(mV, 1) * mV)
        e12 = e12 + 0.5 * (
            v.recip_dyU * (6.0 * uave - _sx(u, -2) * _sx(mU, -1) - _sx(u, 1) * mU) * hU
            + v.recip_dxV * (6.0 * vave - _sy(vv, -2) * _sy(mV, -1) - _sy(vv, 1) * mV) * hV
        )
    return e11, e22, e12


def viscosities(state, e11, e22, e12):
    """veris/dynamics_routines.py:220-268: zeta, eta and replacement pressure."""
    v, s = state.variables, state.settings
    rsq = 1.0 / s.PlasDefCoeff ** 2
    c = v.rAz * e12 ** 2
    c = c + _sx(c, 1)
    c = 0.25 * v.recip_rA * (c + _sy(c, 1))
    dsq = (e11 + e22) ** 2 + rsq * ((e11 - e22) ** 2 + 4.0 * c)
    with np.errstate(invalid="ignore"):
        delta = np.sqrt(dsq)
    zeta = 0.5 * (v.SeaIceStrength * (1 + s.tensileStrFac)) / (delta + s.deltaMin)
    eta = zeta * rsq
    press = (1 * (v.SeaIceStrength * (1 - s.pressReplFac)
                  + 2.0 * zeta * delta * s.pressReplFac / (1 + s.tensileStrFac))
             * (1 - s.tensileStrFac))
    return zeta, eta, press


def stress(state, e11, e22, e12, zeta, eta, press):
    """veris/dynamics_routines.py:271-281 (not used by the EVP loop)."""
    sig11 = 0.5 * (2 * zeta * (e11 + e22) + 2 * eta * (e11 - e22) - press)
    sig22 = 0.5 * (2 * zeta * (e11 + e22) - 2 * eta * (e11 - e22) - press)
    return sig11, sig22, 2.0 * e12 * c_point_to_z_point(state, eta)


def stressdiv(state, sig11, sig22, sig12):
    """veris/dynamics_routines.py:284-303: divergence of the stress tensor."""
    v = state.variables
    a = sig11 * v.dyV
    b = sig12 * v.dxV
    dx = (a - _sx(a, -1) - b + _sy(b, 1)) * v.recip_rAu
    a = sig22 * v.dxU
    b = sig12 * v.dyU
    dy = (a - _sy(a, -1) - b + _sx(b, 1)) * v.recip_rAv
    return dx, dy


def ocean_drag_coeffs(state, u, vv):
    """veris/dynamics_routines.py:21-52: linear ice-ocean drag at C points."""
    v, s = state.variables, state.settings
    dc = np.where(v.fCori < 0, s.waterIceDrag_south, s.waterIceDrag) * s.rhoSea
    du = (u - v.uOcean) * v.maskInU
    dv = (vv - v.vOcean) * v.maskInV
    t = 0.25 * ((du + _sx(du, 1)) ** 2 + (dv + _sy(dv, 1)) ** 2)
    cd = np.where(dc ** 2 * t > s.cDragMin ** 2, dc * np.sqrt(t), s.cDragMin)
    return cd * v.iceMask


def basal_drag_coeffs(state, u, vv):
    """veris/dynamics_routines.py:55-96: basal (landfast) drag at C points."""
    v, s = state.variables, state.settings
    um = u * v.maskInU
    vm = vv * v.maskInV
    t = 0.25 * (um ** 2 + _sx(um, 1) ** 2 + vm ** 2 + _sy(vm, 1) ** 2)
    t = s.basalDragK2 / np.sqrt(t + s.basalDragU0 ** 2)
    hcrit = np.abs(v.R_low) * v.Area / s.basalDragK1
    fac = 10.0
    with np.errstate(over="ignore", invalid="ignore"):
        cb = np.where(v.Area > 0.01,
                      t * np.log(np.exp(fac * (v.hIceMean - hcrit)) + 1.0) * (1.0 / fac)
                      * np.exp(-s.cBasalStar * (1.0 - v.Area)),
                      0.0)
    return cb


def side_drag(state, u, vv):
    """veris/dynamics_routines.py:99-140: lateral (coastal) drag at U and V."""
    v, s = state.variables, state.settings
    sp = 0.5 * np.sqrt((u + _sx(u, 1)) ** 2 + (vv + _sy(vv, 1)) ** 2)
    spU = np.where(v.AreaW > 0, 0.5 * (sp + _sx(sp, -1)), 0)
    spV = np.where(v.AreaS > 0, 0.5 * (sp + _sy(sp, -1)), 0)
    mU = (2 - _sx(v.iceMaskU, -1) - _sx(v.iceMaskU, 1)) * v.iceMaskU
    mV = (2 - _sy(v.iceMaskV, -1) - _sy(v.iceMaskV, 1)) * v.iceMaskV
    if s.use_coastline:
        mU, mV = v.Fu, v.Fv
    return (v.SeaIceMassU * s.sideDragCoeff * mU / (spU + s.sideDragU0),
            v.SeaIceMassV * s.sideDragCoeff * mV / (spV + s.sideDragU0))


# -------------------------------------------------------------------- EVP loop

def evp_subcycle(state, c):
    """One mEVP subcycle, veris/evp_solver.py:21-254, on the carry dict ``c``.

    ``c`` holds u, v, uNm1, vNm1, sigma1, sigma2, sigma12, denom1, denom2,
    EVPcFac, alphaC, alphaZ, betaU, betaV; it is updated in place.  The
    residual branch of the reference (:193-234) reads names the reference
    never defines; ``evp_residuals`` restates what it is meant to compute.
    """
    v, s = state.variables, state.settings
    u, vv = c["u"], c["v"]
    e11, e22, e12 = strainrates(state, u, vv)
    zeta, _eta, press = viscosities(state, e11, e22, e12)
    if s.useAdaptiveEVP:
        aC = np.sqrt(zeta * c["EVPcFac"] / np.maximum(v.SeaIceMassC, 1e-4) * v.recip_rA) * v.iceMask
        aC = np.maximum(aC, s.aEVPalphaMin)
        c["alphaC"] = aC
        c["denom1"] = 1.0 / aC
        c["denom2"] = c["denom1"]
    rev, rrev = 1, 0.25
    ep = e11 + e22
    em = e11 - e22
    div = 2 * zeta * ep - press
    ten = 2 * zeta * em
    shr = 2 * c_point_to_z_point(state, zeta) * e12
    aC = c["alphaC"]
    s1 = (c["sigma1"] * (aC - rev) + div) * c["denom1"] * v.iceMask
    s2 = (c["sigma2"] * (aC - rev) + ten * rrev) * c["denom2"] * v.iceMask
    sig11 = 0.5 * (s1 + s2)
    sig22 = 0.5 * (s1 - s2)
    if s.useAdaptiveEVP:
        aZ = 0.5 * (aC + _sy(aC, -1))
        aZ = 0.5 * (aZ + _sx(aZ, -1))
        c["alphaZ"] = aZ
        c["denom2"] = 1.0 / aZ
    s12 = (c["sigma12"] * (c["alphaZ"] - rev) + shr * rrev) * c["denom2"]
    sdx, sdy = stressdiv(state, sig11, sig22, s12)
    cd = ocean_drag_coeffs(state, u, vv)
    cb = basal_drag_coeffs(state, u, vv)

    lmU = np.where(v.SeaIceMassU != 0, 1, v.SeaIceMassU)
    lmV = np.where(v.SeaIceMassV != 0, 1, v.SeaIceMassV)
    cdW = _sx(cd, -1)
    cdS = _sy(cd, -1)
    sgn = np.sign(v.fCori)
    du = v.uOcean - u
    dv = v.vOcean - vv
    fx = v.WindForcingX + (
        0.5 * (cd + cdW) * s.cosWat * v.uOcean
        - sgn * s.sinWat * 0.5 * (
            cd * 0.5 * (du + _sy(du, 1))
            + cdW * 0.5 * (_sx(du, -1) + _sy(_sx(du, -1), 1))
        ) * lmU) * v.AreaW
    fy = v.WindForcingY + (
        0.5 * (cd + cdS) * s.cosWat * v.vOcean
        + sgn * s.sinWat * 0.5 * (
            cd * 0.5 * (dv + _sx(dv, 1))
            + cdS * 0.5 * (_sy(dv, -1) + _sx(_sy(dv, -1), 1))
        ) * lmV) * v.AreaS
    fvC = v.SeaIceMassC * v.fCori * 0.5 * (vv + _sy(vv, 1))
    fuC = v.SeaIceMassC * v.fCori * 0.5 * (u + _sx(u, 1))
    fx = fx + 0.5 * (fvC + _sx(fvC, -1))
    fy = fy - 0.5 * (fuC + _sy(fuC, -1))

    if s.useAdaptiveEVP:
        c["betaU"] = 0.5 * (aC + _sx(aC, -1))
        c["betaV"] = 0.5 * (aC + _sy(aC, -1))
    bU = c["betaU"] * s.recip_deltatDyn
    bV = c["betaV"] * s.recip_deltatDyn
    bU1 = bU + s.recip_deltatDyn
    bV1 = bV + s.recip_deltatDyn
    dU = v.SeaIceMassU * bU1 + v.AreaW * (0.5 * (cd + cdW) * s.cosWat + 0.5 * (cb + _sx(cb, -1)))
    dV = v.SeaIceMassV * bV1 + v.AreaS * (0.5 * (cd + cdS) * s.cosWat + 0.5 * (cb + _sy(cb, -1)))
    dU = np.where(dU == 0, 1, dU)
    dV = np.where(dV == 0, 1, dV)
    if not s.noSlip:
        sU, sV = side_drag(state, u, vv)
        dU = dU + sU
        dV = dV + sV
    un = v.iceMaskU * (bU * v.SeaIceMassU * u + v.SeaIceMassU * s.recip_deltatDyn * c["uNm1"]
                       + fx + sdx) / dU
    vn = v.iceMaskV * (bV * v.SeaIceMassV * vv + v.SeaIceMassV * s.recip_deltatDyn * c["vNm1"]
                       + fy + sdy) / dV
    un, vn = fill_overlap_uv(state, un, vn)
    c.update(u=un, v=vn, sigma1=s1, sigma2=s2, sigma12=s12)
    return c


def evp_carry(state):
    """The loop carry of veris/evp_solver.py:257-313."""
    v, s = state.variables, state.settings
    shape = v.iceMask.shape
    cfac = (s.deltatDyn * 4 * (np.pi * s.aEvpCoeff) ** 2) if s.useAdaptiveEVP else 0
    d1 = np.full(shape, 1 / s.evpAlpha)
    return dict(u=v.uIce, v=v.vIce, uNm1=v.uIce, vNm1=v.vIce,
                sigma1=v.sigma1, sigma2=v.sigma2, sigma12=v.sigma12,
                denom1=d1, denom2=d1, EVPcFac=cfac,
                alphaC=np.full(shape, float(s.evpAlpha)), alphaZ=np.full(shape, float(s.evpAlpha)),
                betaU=np.full(shape, float(s.evpBeta)), betaV=np.full(shape, float(s.evpBeta)))


def evp_solver(state, n=None):
    """veris/evp_solver.py:257-319: ``nEVPsteps`` subcycles from the state.

    Returns (uIce, vIce, sigma1, sigma2, sigma12).
    """
    c = evp_carry(state)
    for _ in range(state.settings.nEVPsteps if n is None else n):
        evp_subcycle(state, c)
    return c["u"], c["v"], c["sigma1"], c["sigma2"], c["sigma12"]


def evp_residuals(state, n=None):
    """The EVP loop with the residual diagnostics of veris/evp_solver.py:193-234
    as they are meant to work (the reference's branch reads the undefined names
    sigma11/sigma22 and sig11Pm1..., here: the stress components 0.5(s1 +- s2)
    before and after the subcycle).  Per subcycle k, over the interior:

        resSig[k] = sum (d sig11 alphaC iceMask)^2 + (d sig22 alphaC iceMask)^2
                        + (d sigma12 alphaZ)^2
        resU[k]   = sum (iceMaskU d u betaU)^2 + (iceMaskV d v betaV)^2

    Returns (uIce, vIce, sigma1, sigma2, sigma12, resU, resSig)."""
    v, s = state.variables, state.settings
    c = evp_carry(state)
    n = s.nEVPsteps if n is None else n
    resU = np.zeros(n)
    resSig = np.zeros(n)
    I = (slice(s.olx, -s.olx), slice(s.oly, -s.oly))
    for k in range(n):
        u0, v0 = c["u"], c["v"]
        s110 = 0.5 * (c["sigma1"] + c["sigma2"])
        s220 = 0.5 * (c["sigma1"] - c["sigma2"])
        s120 = c["sigma12"]
        evp_subcycle(state, c)
        s11 = 0.5 * (c["sigma1"] + c["sigma2"])
        s22 = 0.5 * (c["sigma1"] - c["sigma2"])
        d11 = (s11 - s110) * c["alphaC"] * v.iceMask
        d22 = (s22 - s220) * c["alphaC"] * v.iceMask
        d12 = (c["sigma12"] - s120) * c["alphaZ"]
        du = v.iceMaskU * (c["u"] - u0) * c["betaU"]
        dv = v.iceMaskV * (c["v"] - v0) * c["betaV"]
        resSig[k] = (d11 ** 2 + d22 ** 2 + d12 ** 2)[I].sum()
        resU[k] = (du ** 2 + dv ** 2)[I].sum()
    return c["u"], c["v"], c["sigma1"], c["sigma2"], c["sigma12"], resU, resSig


def freedrift_solver(state):
    """veris/freedrift_solver.py:5-62: ice velocities without internal stress."""
    v, s = state.variables, state.settings
    tauXc = 0.5 * (v.WindForcingX + _sx(v.WindForcingX, 1))
    tauYc = 0.5 * (v.WindForcingY + _sy(v.WindForcingY, 1))
    mIceCor = s.rhoIce * v.hIceMean * v.fCori
    uOc = 0.5 * (v.uOcean + _sx(v.uOcean, 1))
    vOc = 0.5 * (v.vOcean + _sy(v.vOcean, 1))
    rhsX = -tauXc - mIceCor * vOc
    rhsY = -tauYc + mIceCor * uOc
    t1 = rhsX ** 2 + rhsY ** 2
    w1 = t1 > 0
    rhsN = np.where(w1, np.sqrt(rhsX ** 2 + rhsY ** 2), 0)
    rhsA = np.where(w1, np.arctan2(rhsY, rhsX), 0)
    t1 = 1 / (np.where(v.fCori < 0, s.waterIceDrag_south, s.waterIceDrag) * s.rhoSea)
    t2 = t1 ** 2 * mIceCor ** 2
    t3 = t1 ** 2 * rhsN ** 2
    t4 = t2 ** 2 + 4 * t3
    with np.errstate(invalid="ignore"):
        solN = np.where(t3 > 0, np.sqrt(0.5 * (np.sqrt(t4) - t2)), 0)
    t1 = 1 / t1
    t2 = t1 * solN ** 2
    t3 = mIceCor * solN
    t4 = t2 ** 2 + t3 ** 2
    solA = np.where(t4 > 0, rhsA - np.arctan2(t3, t2), 0)
    uC = uOc - solN * np.cos(solA)
    vC = vOc - solN * np.sin(solA)
    u = 0.5 * (_sx(uC, -1) + uC) * v.iceMaskU
    vv = 0.5 * (_sy(vC, -1) + vC) * v.iceMaskV
    return u, vv


def bulkf_formula_lanl(state, uw, vw, ta, qa, tsf, ocn_mask):
    """veris/heat_flux_MITgcm.py:5-123: bulk fluxes over open ocean ->
    (flwupa, flha, fsha, df0dT, ust, vst, evp, ssq, dEvdT)."""
    s = state.settings
    ht, zref, zice = 2.0, 10.0, 0.0005
    aln = np.log(ht / zref)
    czol = zref * s.karman * s.grav
    lath = np.ones_like(ocn_mask) * s.latvap
    us = np.sqrt(uw * uw + vw * vw)
    usm = np.maximum(us, 1.0)
    t0 = ta * (1.0 + s.zvir * qa)
    ssq = 3.797915 * np.exp(lath * (7.93252e-6 - 2.166847e-3 / tsf)) / 1013.0
    deltap = ta - tsf + s.gamma_blk * ht
    delq = qa - ssq
    rdn = s.karman / np.log(zref / zice)
    rhn = ren = rdn
    ustar = rdn * usm
    tstar = rhn * deltap
    qstar = ren * delq
    for _ in range(5):
        huol = czol / ustar ** 2 * (tstar / t0 + qstar / (1.0 / s.zvir + qa))
        huol = np.minimum(np.abs(huol), 10.0) * np.sign(huol)
        stable = 0.5 + 0.5 * np.sign(huol)
        xsq = np.maximum(np.sqrt(np.abs(1.0 - 16.0 * huol)), 1.0)
        x = np.sqrt(xsq)
        psimh = -5.0 * huol * stable + (1.0 - stable) * (
            2.0 * np.log(0.5 * (1.0 + x)) + 2.0 * np.log(0.5 * (1.0 + xsq)) - 2.0 * np.arctan(x) + np.pi * 0.5)
        psixh = -5.0 * huol * stable + (1.0 - stable) * (2.0 * np.log(0.5 * (1.0 + xsq)))
        rd = rdn / (1.0 + rdn * (aln - psimh) / s.karman)
        rh = rhn / (1.0 + rhn * (aln - psixh) / s.karman)
        re = rh
        ustar = rd * usm
        qstar = re * delq
        tstar = rh * deltap
    csha = s.rhoAir * s.cpdair * us * rh * rd
    clha = s.rhoAir * lath * us * re * rd
    fsha = csha * deltap
    flha = clha * delq
    evp = -flha / lath
    flwupa = s.ocean_emissivity * s.stefBoltz * tsf ** 4
    dflwupdt = 4.0 * s.ocean_emissivity * s.stefBoltz * tsf ** 3
    devdt = clha * ssq * 2.166847e-3 / (tsf * tsf)
    dflhdt = -lath * devdt
    dfshdt = -csha
    df0dt = -dflwupdt + dfshdt + dflhdt
    cdn = 2.7e-3 / usm + 0.142e-3 + 0.0764e-3 * usm
    ust = s.rhoAir * cdn * us * uw
    vst = s.rhoAir * cdn * us * vw
    return flwupa, flha, fsha, df0dt, ust, vst, evp, ssq, devdt


def IceVelocities(state):
    """veris/dynsolver.py:87-102 with the EVP solver selected."""
    if not state.settings.useEVP:
        raise NotImplementedError("only the EVP solver is part of the step")
    return evp_solver(state)


def OceanStressUV(state):
    """veris/ocean_stress.py:8-40: ice-ocean stress at U and V, halo-filled."""
    v, s = state.variables, state.settings
    cd = ocean_drag_coeffs(state, v.uIce, v.vIce)
    sinW = np.sin(np.deg2rad(s.waterTurnAngle))
    cosW = np.cos(np.deg2rad(s.waterTurnAngle))
    du = v.uIce - v.uOcean
    dv = v.vIce - v.vOcean
    duC = 0.5 * (du + _sx(du, 1))
    dvC = 0.5 * (dv + _sy(dv, 1))
    sgn = np.sign(v.fCori)
    a = cd * dvC
    su = 0.5 * (cd + _sx(cd, -1)) * cosW * du - sgn * sinW * 0.5 * (a + _sy(a, -1))
    b = cd * duC
    sv = 0.5 * (cd + _sy(cd, -1)) * cosW * dv + sgn * sinW * 0.5 * (b + _sx(b, -1))
    return fill_overlap_uv(state, su, sv)


# ------------------------------------------------------------------- advection

def limiter(Cr):
    """veris/advection.py:170-175: superbee."""
    return np.maximum(0, np.maximum(np.minimum(1, 2 * Cr), np.minimum(2, Cr)))


def _slope_ratio(Rjm, Rj, Rjp, trans, CrMax):
    cr = np.where(trans > 0, Rjm, Rjp)
    with np.errstate(divide="ignore", invalid="ignore"):
        cr = np.where(np.abs(Rj) * CrMax > np.abs(cr), cr / Rj, np.sign(cr) * CrMax * np.sign(Rj))
    return limiter(cr)


def calc_ZonalFlux(state, field, uTrans):
    """veris/advection.py:94-129: limited flux through the U faces."""
    v, s = state.variables, state.settings
    m = v.iceMaskU * v.maskInU
    cfl = np.abs(v.uIce * s.deltatTherm * v.recip_dxC)
    Rjp = (field[3:, :] - field[2:-1, :]) * m[3:, :]
    Rj = (field[2:-1, :] - field[1:-2, :]) * m[2:-1, :]
    Rjm = (field[1:-2, :] - field[:-3, :]) * m[1:-2, :]
    t = uTrans[2:-1, :]
    cr = _slope_ratio(Rjm, Rj, Rjp, t, s.CrMax)
    F = np.zeros(v.iceMask.shape)
    F[2:-1, :] = (t * (field[2:-1, :] + field[1:-2, :]) * 0.5
                  - np.abs(t) * ((1 - cr) + cfl[2:-1, :] * cr) * Rj * 0.5)
    return fill_overlap(state, F)


def calc_MeridionalFlux(state, field, vTrans):
    """veris/advection.py:132-167: limited flux through the V faces."""
    v, s = state.variables, state.settings
    m = v.iceMaskV * v.maskInV
    cfl = np.abs(v.vIce * s.deltatTherm * v.recip_dyC)
    Rjp = (field[:, 3:] - field[:, 2:-1]) * m[:, 3:]
    Rj = (field[:, 2:-1] - field[:, 1:-2]) * m[:, 2:-1]
    Rjm = (field[:, 1:-2] - field[:, :-3]) * m[:, 1:-2]
    t = vTrans[:, 2:-1]
    cr = _slope_ratio(Rjm, Rj, Rjp, t, s.CrMax)
    F = np.zeros(v.iceMask.shape)
    F[:, 2:-1] = (t * (field[:, 2:-1] + field[:, 1:-2]) * 0.5
                  - np.abs(t) * ((1 - cr) + cfl[:, 2:-1] * cr) * Rj * 0.5)
    return fill_overlap(state, F)


def calc_Advection(state, field):
    """veris/advection.py:28-91, extensive fields (the reference's default;
    its non-extensive branch reads variables it never defines)."""
    v, s = state.variables, state.settings
    if not s.extensiveFld:
        raise NotImplementedError("non-extensive advection is not defined by the reference")
    uT = v.uIce * (v.dyG * v.iceMaskU)
    vT = v.vIce * (v.dxG * v.iceMaskV)
    F = calc_ZonalFlux(state, field, uT)
    f = field - s.deltatTherm * v.maskInC * v.recip_rA * (_sx(F, 1) - F)
    G = calc_MeridionalFlux(state, f, vT)
    f = f - s.deltatTherm * v.maskInC * v.recip_rA * (_sy(G, 1) - G)
    return f * v.iceMask


def Advection(state):
    """veris/advection.py:15-25."""
    v = state.variables
    return (calc_Advection(state, v.hIceMean), calc_Advection(state, v.hSnowMean),
            calc_Advection(state, v.Area))


def clean_up_advection(state):
    """veris/clean_up.py:5-39."""
    v, s = state.variables, state.settings
    os_h = np.maximum(-v.hIceMean, 0)
    os_s = np.maximum(-v.hSnowMean, 0)
    h = np.maximum(v.hIceMean, 0)
    hs = np.maximum(v.hSnowMean, 0)
    A = np.maximum(v.Area, 0)
    thin = h <= s.hIce_min
    h = h * ~thin
    hs = hs * ~thin
    T = np.where(thin, s.celsius2K, v.TSurf)
    A = np.where((h == 0) & (hs == 0), 0, A)
    A = np.where((h > 0) | (hs > 0), np.maximum(A, s.Area_min), A)
    return h, hs, A, T, os_h, os_s


def ridging(state):
    """veris/clean_up.py:42-47."""
    return np.minimum(state.variables.Area, 1)


# --------------------------------------------------------------- thermodynamics

def solve4temp(state, hIceActual, hSnowActual, TSurfIn, TempFrz):
    """veris/solve4temp.py:5-174: surface temperature by 6 Newton steps."""
    v, s = state.variables, state.settings
    aa1, aa2, bb1 = 2663.5, 12.537, 0.622
    bb2 = 1 - bb1
    P = 100000
    cc0 = 10 ** aa2
    cc1 = cc0 * aa1 * bb1 * P * np.log(10)
    cc2 = cc0 * bb2
    d1 = s.dalton * s.cpAir * s.rhoAir
    d1i = s.dalton * s.lhSublim * s.rhoAir
    Tmelt = s.celsius2K
    SurfMeltTemp = Tmelt + s.wetAlbTemp
    T = TSurfIn
    lwc = np.maximum(s.minLWdown, v.LWdown)
    Ta = np.maximum(s.celsius2K + s.minTAir, v.ATemp)
    ug = np.maximum(s.wSpeedMin, v.wSpeed)
    ice = hIceActual > 0
    snow = hSnowActual > 0
    d3 = np.where(snow, s.snowEmiss, s.iceEmiss) * s.stefBoltz
    lw = np.where(snow, s.snowEmiss, s.iceEmiss) * lwc

    aI = np.where(ice, s.dryIceAlb, 0)
    aS = np.where(ice, s.drySnowAlb, 0)
    wet = (hIceActual > 0) & (T >= SurfMeltTemp)
    aI = np.where(wet, s.wetIceAlb, aI)
    aS = np.where(wet, s.wetSnowAlb, aS)
    south = (hIceActual > 0) & (v.fCori < 0)
    aI = np.where(south, s.dryIceAlb_south, aI)
    aS = np.where(south, s.drySnowAlb_south, aS)
    wet_s = (hIceActual > 0) & (v.fCori < 0) & (T >= SurfMeltTemp)
    aI = np.where(wet_s, s.wetIceAlb_south, aI)
    aS = np.where(wet_s, s.wetSnowAlb_south, aS)
    alb = np.where(ice, aI + hSnowActual / s.hCut * (aS - aI), 0)
    alb = np.where(hSnowActual > s.hCut, aS, alb)
    alb = np.where(hSnowActual == 0, aI, alb)

    pen = np.where(ice, s.shortwave * np.exp(-1.5 * hIceActual), 0)
    pen = np.where(snow, 0, pen)
    penSW = np.where(ice, -(1 - alb) * pen * v.SWdown, 0)
    absSW = np.where(ice, (1 - alb) * (1 - pen) * v.SWdown, 0)
    with np.errstate(divide="ignore", invalid="ignore"):
        k = np.where(ice, s.iceConduct * s.snowConduct
                     / (s.snowConduct * hIceActual + s.iceConduct * hSnowActual), 0)

    def fluxes(t1):
        t2 = t1 * t1
        t3 = t2 * t1
        t4 = t2 * t2
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            svp = 10 ** (-aa1 / t1 + aa2)
            qs = np.where(ice, bb1 * svp / (P - (1 - bb1) * svp), 0)
            c3 = 10 ** (aa1 / t1)
            dqs = np.where(ice, cc1 * c3 / ((cc2 - c3 * P) ** 2 * t2), 0)
        Fc = np.where(ice, k * (TempFrz - t1), 0)
        Flh = np.where(ice, d1i * ug * (qs - v.aqh), 0)
        Flw = np.where(ice, t4 * d3, 0)
        Fs = np.where(ice, d1 * ug * (t1 - Ta), 0)
        Fia = np.where(ice, (-lw - absSW + Flw + Fs + Flh), 0)
        dF = np.where(ice, 4 * d3 * t3 + d1 * ug + d1i * ug * dqs, 0)
        return Fc, Flh, Fia, dF

    for _ in range(6):
        Fc, Flh, Fia, dF = fluxes(T)
        with np.errstate(divide="ignore", invalid="ignore"):
            T = np.where(ice, T + (Fc - Fia) / (k + dF), 0)
        T = np.minimum(T, Tmelt)
        T = np.maximum(T, s.celsius2K + s.minTIce)
    Fc, Flh, Fia, dF = fluxes(T)
    up = Fc > 0
    return (np.where(ice, T, TSurfIn), np.where(up, Fc, 0), np.where(up, 0, Fia),
            penSW, np.where(ice, Flh / s.lhSublim, 0))


def Growth(state):
    """veris/growth.py:8-397: thermodynamic growth and the ocean budgets."""
    v, s = state.variables, state.settings
    qi = 1 / (s.rhoIce * s.lhFusion)
    qs = 1 / (s.rhoSnow * s.lhFusion)
    noIce = (v.hIceMean == 0) | (v.Area == 0)
    h0 = v.hIceMean * ~noIce
    hs0 = v.hSnowMean * ~noIce
    A0 = v.Area * ~noIce
    isIce = h0 > 0
    regA = np.sqrt(A0 ** 2 + s.Area_reg)
    rregA = 1 / regA
    hIa = np.where(isIce, h0 * rregA, 0)
    rhIa = A0 / np.sqrt(h0 ** 2 + s.hIce_reg)
    hSa = np.where(isIce, hs0 * rregA, 0)
    hIa = np.maximum(hIa, 0.05)

    TempFrz = s.tempFrz + s.dtempFrz_dS * v.ocSalt + s.celsius2K
    n = s.nITC
    T_sum = np.zeros_like(h0)
    Fio_sum = np.zeros_like(h0)
    Fia_sum = np.zeros_like(h0)
    pen_sum = np.zeros_like(h0)
    for l in range(n):
        pFac = (2 * (l + 1) - 1) * s.recip_nITC
        out = solve4temp(state, hIa * pFac, hSa * pFac, v.TSurf, TempFrz)
        T_sum = T_sum + out[0]
        Fio_sum = Fio_sum + out[1]
        Fia_sum = Fia_sum + out[2]
        pen_sum = pen_sum + out[3]
    TSurf = T_sum * s.recip_nITC
    Fio = Fio_sum * s.recip_nITC * A0
    Fia = Fia_sum * s.recip_nITC * A0
    pen = pen_sum * s.recip_nITC * A0

    cold = (A0 > 0) & (T_sum / n < s.celsius2K)
    snowAcc = np.where(cold, v.snowfall + v.precip, v.snowfall) * s.rhoFresh2rhoSnow
    rainToSea = np.where(cold, 0, v.precip)
    snowAccOverIce = snowAcc * A0 * s.deltatTherm

    gUnder = Fio * qi
    gUnder = np.where(A0 == 0, 0, gUnder)
    potMeltRate = -Fia * qs
    potMelt = potMeltRate * s.deltatTherm
    allMelt = potMelt >= hs0
    meltRate = np.where(allMelt, np.where(allMelt, hs0, potMelt) * s.recip_deltatTherm, potMeltRate)
    toSnow = np.where(allMelt, -hs0 * s.recip_deltatTherm / qs, Fia)
    Fia = Fia - toSnow
    gSurf = Fia * qi
    gNet = (gUnder + gSurf) * rregA

    t0 = 0.4
    t1 = 7 / t0
    t2 = s.stantonNr * s.uStarBase * s.rhoSea * s.cpWater
    sst = np.maximum(v.theta, TempFrz)
    mltf = 1 + (s.McPheeTaperFac - 1) / (1 + np.exp((A0 - t0) * t1))
    gML = -t2 * (sst - TempFrz) * mltf * qi
    gOW = qi * v.Qnet

    dh = gNet * A0 + gOW * (1 - A0) + gML
    dhs = (snowAcc - meltRate) * A0
    half_rh = 0.5 * rhIa
    dA_oa = half_rh * gOW * (1 - A0)
    grow = (gOW > 0) & ((A0 > 0) | (dh > 0))
    dA_oa = np.where(grow, gOW * (1 - A0), dA_oa)
    dA_oa = np.where(grow & (v.fCori < 0), dA_oa * s.recip_h0_south, dA_oa * s.recip_h0)
    dA_oi = np.where(gML <= 0, half_rh * gML, 0)
    dA_ia = np.where((gNet <= 0) & (h0 > 0), half_rh * gNet * A0, 0)
    dA = dA_oa + dA_oi + dA_ia

    A = A0 + dA * v.iceMask * s.deltatTherm
    h = h0 + dh * v.iceMask * s.deltatTherm
    hs = hs0 + dhs * v.iceMask * s.deltatTherm
    A = np.clip(A, 0, 1)
    h = np.maximum(h, 0)
    hs = np.maximum(hs, 0)
    gone = (h == 0) | (A == 0)
    A = A * ~gone
    hs = hs * ~gone
    h = h * ~gone
    hsub = (hs * s.rhoSnow + h * s.rhoIce) * s.recip_rhoSea
    flood = np.maximum(0, hsub - h)
    h = h + flood
    hs = hs - flood * s.rhoIce2rhoSnow
    rh = 1 / np.sqrt(h ** 2 + s.hIce_reg)

    Qsw = pen * A0 + v.Qsw * (1 - A0)
    dH = h - h0
    melted = hs0 + snowAccOverIce - hs
    E_ice = dH / qi
    E_out = (A0 * (Fia + Fio + pen) + (1 - A0) * v.Qnet) * s.deltatTherm
    Qnet = (E_out - E_ice) * s.recip_deltatTherm
    with np.errstate(divide="ignore", invalid="ignore"):
        fw_ice = -dH * s.rhoIce2rhoFresh * np.where((v.ocSalt > 0) & (v.ocSalt > s.saltIce_ref),
                                                     (1 - s.saltIce_ref / v.ocSalt), 1)
    salt_ref = np.minimum(s.saltIce_ref, v.ocSalt)
    saltflux = (dH + v.os_hIceMean) * salt_ref * v.iceMask * s.rhoIce * s.recip_deltatTherm
    fw_snow = melted / s.rhoFresh2rhoSnow
    EmPmR = (v.iceMask * ((-v.evap - v.precip) * (1 - A0) - rainToSea * A0 - v.runoff
                          - (fw_ice + fw_snow) / s.deltatTherm) * s.rhoFresh
             + v.iceMask * (v.os_hIceMean * s.rhoIce + v.os_hSnowMean * s.rhoSnow)
             * s.recip_deltatTherm)
    forc_salt = EmPmR * v.ocSalt / s.rhoFresh + saltflux
    load = h * s.rhoIce + hs * s.rhoSnow
    return h, hs, A, TSurf, EmPmR, forc_salt, Qsw, Qnet, load, pen, rh


# ------------------------------------------------------------------------ step

STEP_OUTPUTS = (
    ("SeaIceMass", ("SeaIceMassC", "SeaIceMassU", "SeaIceMassV")),
    ("AreaWS", ("AreaW", "AreaS")),
    ("WindForcingXY", ("WindForcingX", "WindForcingY")),
    ("SeaIceStrength", ("SeaIceStrength",)),
    ("IceVelocities", ("uIce", "vIce", "sigma1", "sigma2", "sigma12")),
    ("OceanStressUV", ("OceanStressU", "OceanStressV")),
    ("Advection", ("hIceMean", "hSnowMean", "Area")),
    ("clean_up_advection", ("hIceMean", "hSnowMean", "Area", "TSurf", "os_hIceMean",
                            "os_hSnowMean")),
    ("ridging", ("Area",)),
    ("Growth", ("hIceMean", "hSnowMean", "Area", "TSurf", "EmPmR", "forc_salt_surface_ice",
                "Qsw", "Qnet", "SeaIceLoad", "IcePenetSW", "recip_hIceMean")),
)
FILLED_AFTER_GROWTH = ("hIceMean", "hSnowMean", "Area", "forc_salt_surface_ice", "Qnet")


def step(state, record=None):
    """One sea-ice step in the order of the reference setup's step
    (veris/setup/seaice_global_4deg/seaice_global_4deg.py:878-932): dynamics
    preparation, EVP, ocean stress, advection, clean-up, ridging, growth and
    the final halo fills.  All five EVP results, stresses included, are stored
    back into the state.  ``record(name, outputs)`` sees every call.
    """
    v = state.variables
    g = globals()
    for name, outs in STEP_OUTPUTS:
        vals = g[name](state)
        if not isinstance(vals, tuple):
            vals = (vals,)
        vals = tuple(np.array(x, dtype=np.float64) for x in vals)
        if record is not None:
            record(name, dict(zip(outs, vals)))
        for n, x in zip(outs, vals):
            setattr(v, n, x)
    for n in FILLED_AFTER_GROWTH:
        x = fill_overlap(state, getattr(v, n).copy())
        if record is not None:
            record("fill_overlap", {n: x})
        setattr(v, n, x)
    return state
