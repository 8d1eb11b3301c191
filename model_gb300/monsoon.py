"""Monsoon-depression initial state: the reference's ITCZ-shear basic state and
axisymmetric vortex, restated in numpy.

The reference builds this state in initialize_basic_state_ITCZ_shear2
(data_initializer.cpp:298-568) and initialize_vortex (:862-1064) of its
parallel build.  The steps, in the reference's order:

  1. the 20N/88E sounding (get_base_state_from_20_88, :1699-1745) interpolated
     to the model levels (vert_interpolate_1d, interpolate.cpp:562-640) and
     the column state built from it (initialize_vertical_basic_state2,
     initializer.cpp:858-928);
  2. a strip of relative vorticity between 18N and 21N up to 17 km
     (create_horizontal_shear_zone, :83-139) and its streamfunction
     (get_stream_function, :145-169, by run_laplacian_solver,
     laplacian.cpp:181-245: FFT in x, tridiagonal solve in y);
  3. a zonal wind u(z) + 3 m/s with the shear of create_vertical_shear_profile
     (:195-221), plus the rotational wind of the streamfunction;
  4. pressure in geostrophic balance with u (get_pressure_from_winds,
     :229-255), the 20N/88E column subtracted (subtract_base_state, :264-274),
     theta in hydrostatic balance with it (hydrostatic_balance, :283-289), and
     the pressure made non-dimensional;
  5. basic-state vapour from a latitude-dependent relative humidity;
  6. the whole wind/pressure/theta pass repeated for the final vorticity
     (hor_shear - 1e-4), which also recomputes the pressure on top of the
     first pass's non-dimensional values in the rows that
     get_pressure_from_winds does not write (row j = 0, column i = NX-1);
  7. top/bottom copies and the basic-state vertical velocity from continuity
     (init_basic_state_vertical_velocity, initializer.cpp:1113-1135);
  8. the vortex: a warm-over-cold theta anomaly, its hydrostatic geopotential
     and the gradient wind, interpolated from radius to the grid and
     staggered (initialize_vortex).

One deviation, forced: create_vertical_shear_profile is called with ktrop = 37,
which overruns its arrays when NZ <= 38 (the reference's 32-level
configuration among them).  ktrop is clamped to NZ - 2 here; with NZ >= 39 the
restatement follows the reference exactly.

Pinned against the reference itself (oracle/ref/itcz_harness.cpp, fixture
tests/golden/itcz_*.npz).
"""
from __future__ import annotations

import numpy as np

RD, CP, CV, P0, GRAV = 287.0, 1004.0, 717.0, 100000.0, 9.8
PRESSFC = 100200.0
TRIGPI = 3.14159265358979324
FC = 7.292e-5
MPD = 111000.0
LOWER_LAT = -89.462997

# get_base_state_from_20_88 (data_initializer.cpp:1699-1745): theta (K),
# vapour (kg/kg) and height (m) of the reference's 20N/88E column.  Data the
# initial state is defined by, so kept as the reference gives it.
_SOUNDING_TB = np.array([
    301.3688257116, 301.8163590723, 302.3725230915, 303.5396454461, 304.4779570865, 305.4938954838,
    306.6227667893, 307.8911249353, 309.2454008827, 310.6936441680, 312.2381766112, 315.4918989755,
    318.7967845618, 321.8109652832, 325.3755268822, 330.0211783507, 334.5667331740, 339.1455453915,
    343.9030848237, 348.2139891673, 352.0680543027, 353.6331293068, 355.0080137497, 356.5539533635,
    358.7368337136, 362.1445309838, 373.4121328070, 429.4978633148, 492.4724739660, 593.3140366746,
    681.8870810434, 857.2924158974, 967.5530849371, 1092.1733790195, 1319.2834107809, 1518.7488915123,
    1882.5817225223])
_SOUNDING_QB = np.array([
    0.0199446990, 0.0190561418, 0.0181378907, 0.0171884018, 0.0164599732, 0.0157072981,
    0.0149655603, 0.0142159289, 0.0134605601, 0.0126884429, 0.0119014775, 0.0103284225,
    0.0088135030, 0.0074222058, 0.0062207775, 0.0051422818, 0.0039585675, 0.0027820404,
    0.0017543257, 0.0009854162, 0.0004371278, 0.0002502617, 0.0001286210, 0.0000598493,
    0.0000244848, 0.0000085451, 0.0000032968, 0.0000025111, 0.0000024027, 0.0000024293,
    0.0000025173, 0.0000026986, 0.0000028049, 0.0000029210, 0.0000031283, 0.0000033081,
    0.0000036400])
_SOUNDING_Z = np.array([
    -4.9309824095, 220.0563275839, 449.7083182255, 684.3637424527, 924.2080450767, 1169.5747824156,
    1420.7582630933, 1678.1441041335, 1942.1632221482, 2213.2407713351, 2491.8242119209, 3073.6699679147,
    3691.7716591048, 4350.8611958576, 5056.6653728972, 5819.2277164608, 6649.4016027568, 7560.0781719656,
    8569.3345586917, 9701.5591376725, 10992.8973225474, 11714.3712557337, 12499.8515755171, 13360.3068109264,
    14318.2241373647, 15405.7570490178, 16685.1606511117, 18733.0547480514, 20752.9602378743, 23947.3420385707,
    26561.1613501294, 31151.8561242708, 33573.3309380886, 35905.4984772108, 39575.7896964869, 42588.1612632421,
    47859.5785629266])


# ---------------------------------------------------------------------------
# grid and column helpers
# ---------------------------------------------------------------------------
def _coords(n: int, start: float, step: float) -> np.ndarray:
    """outLons / outLats of setup_coordinates (initializer.cpp:1948-1967):
    a start value then a running sum of equal steps."""
    a = np.full(n, step)
    a[0] = start
    return np.cumsum(a)


def _nearest(values: np.ndarray, x: float) -> int:
    """get_point_from_lat / _lon / _height (util.cpp:480-545): the first
    index whose value is not below x, or the one before it if that is
    closer.  x must lie inside the array (the reference reads index -1 or
    stops the program otherwise)."""
    p = 0
    while x > values[p]:
        p += 1
        if p >= values.size:
            raise ValueError(f"{x} lies beyond the grid")
    if p == 0:
        raise ValueError(f"{x} lies below the grid")
    return p - 1 if abs(values[p - 1] - x) < abs(values[p] - x) else p


def _cubic(y0, y1, y2, y3, mu):
    """CubicInterpolate2 (interpolate.cpp:1403-1416)."""
    f0p = (y2 - y0) / 2
    f1p = (y3 - y1) / 2
    a = 2 * y1 - 2 * y2 + f0p + f1p
    b = -3 * y1 + 3 * y2 - 2 * f0p - f1p
    return a * mu * mu * mu + b * mu * mu + f0p * mu + y1


def _interp_column(z_in: np.ndarray, v_in: np.ndarray, z_out: np.ndarray) -> np.ndarray:
    """vert_interpolate_1d(nzIn, nzOut, ...) (interpolate.cpp:562-640):
    cubic inside the data, one-sided ends, linear below the lowest point."""
    n_in = z_in.size
    out = np.zeros(z_out.size)
    count = 0
    k = 0
    while k < z_out.size:
        z = z_out[k]
        if z > z_in[count] and z <= z_in[count + 1]:
            mu = (z - z_in[count]) / (z_in[count + 1] - z_in[count])
            if count != 0 and count < n_in - 2:
                out[k] = _cubic(v_in[count - 1], v_in[count], v_in[count + 1], v_in[count + 2], mu)
            elif count == 0:
                out[k] = _cubic(2 * v_in[0] - v_in[1], v_in[0], v_in[1], v_in[2], mu)
            else:
                out[k] = _cubic(v_in[count - 1], v_in[count], v_in[count + 1], 2 * v_in[count + 1] - v_in[count],
                                mu)
        elif z < z_in[0]:
            mu = (z - z_in[0]) / (z_in[1] - z_in[0])
            out[k] = v_in[0] * (1 - mu) + v_in[1] * mu  # LinearInterpolate (:1454-1457)
        elif z > z_in[n_in - 1]:
            break
        elif z == z_in[count]:
            out[k] = v_in[count]
        else:
            count += 1
            continue
        k += 1
    return out


def _qvsat(temperature, pressure):
    """get_QV_Sat (initializer.cpp:1387-1392)."""
    esl = 611.2 * np.exp(17.67 * (temperature - 273.15) / (temperature - 29.65))
    return 0.62197 * esl / (pressure - esl)


def sounding_20n_88e(zu: np.ndarray):
    """tb, qb on the model levels (get_base_state_from_20_88)."""
    tb = _interp_column(_SOUNDING_Z, _SOUNDING_TB, zu)
    qb = _interp_column(_SOUNDING_Z, _SOUNDING_QB, zu)
    tb[0], tb[-1] = tb[1], tb[-2]
    qb[0], qb[-1] = qb[1], qb[-2]
    return tb, qb


def column_state(tb: np.ndarray, qb: np.ndarray, zsu: np.ndarray):
    """tbv, pib, rhou, rhow of initialize_vertical_basic_state2
    (initializer.cpp:858-928, stretched-grid branch)."""
    nz = tb.size
    tbv = tb * (1.0 + 0.61 * qb)
    pisfc = (PRESSFC / P0) ** (RD / CP)
    pib = np.zeros(nz)
    pib[1] = pisfc - GRAV * (zsu[1] - 0) / (CP * tbv[1])
    pib[0] = pisfc + GRAV * (0 - zsu[0]) / (CP * tbv[0])
    for k in range(2, nz):
        pib[k] = pib[k - 1] - GRAV * (zsu[k] - zsu[k - 1]) / (CP * (0.5 * (tbv[k] + tbv[k - 1])))
    rhou = P0 * pib ** (CV / RD) / (RD * tbv)
    rhow = np.zeros(nz)
    rhow[1:] = 0.5 * (rhou[1:] + rhou[:-1])
    rhow[0] = rhow[1]
    tbv[0], tbv[-1] = tbv[1], tbv[-2]
    pib[0], pib[-1] = pib[1], pib[-2]
    return tbv, pib, rhou, rhow


def _cos_profile(pl, ph, frac, shift):
    """cos_profile (util.cpp:740-749): a cosine segment on frac in [0, 1]."""
    frac = np.asarray(frac, dtype=np.float64)
    v = np.cos(pl * 2 * TRIGPI + (ph - pl) * 2 * TRIGPI * frac) + shift
    return np.where((frac >= 0) & (frac <= 1.0), v, 0.0)


# ---------------------------------------------------------------------------
# the basic state
# ---------------------------------------------------------------------------
class _Grid:
    def __init__(self, nx, ny, nz, dx, dy, dz, corner_lat, corner_lon):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dx, self.dy, self.dz = dx, dy, dz
        # uniform levels (height_lowest_level = dz: stretched_grid's c1 = 1, c2 = 0)
        self.zsu = (np.arange(nz, dtype=np.float64) - 0.5) * dz
        self.zsw = (np.arange(nz, dtype=np.float64) - 1.0) * dz
        self.lats = _coords(ny, LOWER_LAT + corner_lat + dy / MPD, dy / MPD)
        self.lons = _coords(nx, 0.0 + corner_lon + dx / MPD - 0.0, dx / MPD)
        self.f = 2 * FC * np.sin(self.lats * TRIGPI / 180.)


def _shear_zone(g: _Grid, amp: float, lat0=18.0, lat1=21.0, top_height=17000.0) -> np.ndarray:
    """create_horizontal_shear_zone(amp, lat0, lat1, -1, -1, top_height, 0)."""
    lo, hi = _nearest(g.lats, lat0), _nearest(g.lats, lat1)
    ktop = _nearest(g.zsu, top_height)
    vort = np.zeros((g.nx, g.ny, g.nz))
    j = np.arange(lo, hi)
    fz = 0.5 * _cos_profile(-0.1, 0.5, (g.zsu[:ktop] - 0) / (top_height - 0), 1.0)
    fy = _cos_profile(-0.5, 0.5, (j - lo).astype(np.float64) / float(hi - lo), 1)
    mult = (fz[None, :] * 0.5) * fy[:, None]  # [j][k]
    vort[:, lo:hi, :ktop] = amp * mult[None, :, :]
    return vort


def _streamfunction(g: _Grid, vort: np.ndarray) -> np.ndarray:
    """get_stream_function: per level, run_laplacian_solver (FFT in x,
    tridiagonal in y with the reference's coefficients; the last row keeps
    the transformed right-hand side, as the reference's back substitution
    starts from it)."""
    nx, ny = g.nx, g.ny
    kw = np.array([2 * TRIGPI * i / nx if i < nx // 2 else 2 * TRIGPI * (nx - i) / nx for i in range(nx)])
    a = 1. / (g.dy * g.dy)
    c = 1. / (g.dy * g.dy)
    b = 2. * (np.cos(kw) - 1.) / (g.dx * g.dx) - c - a  # [i]
    out = np.zeros_like(vort)
    for k in range(g.nz):
        spec = np.fft.fft(vort[:, :, k], axis=0) / nx  # [i][j]
        for part in (0, 1):
            x = spec.real.copy() if part == 0 else spec.imag.copy()
            P = np.zeros((nx, ny + 1))
            Q = np.zeros((nx, ny + 1))
            for j in range(ny):
                denom = b + a * P[:, j]
                P[:, j + 1] = -c / denom
                Q[:, j + 1] = (x[:, j] - a * Q[:, j]) / denom
            for j in range(ny - 2, -1, -1):
                x[:, j] = P[:, j + 1] * x[:, j + 1] + Q[:, j + 1]
            if part == 0:
                re = x
            else:
                im = x
        out[:, :, k] = (np.fft.ifft(re + 1j * im, axis=0) * nx).real
    return out


def _shear_profile(g: _Grid, top: float, bot: float, midlev: float, ktrop: int) -> np.ndarray:
    """create_vertical_shear_profile(top, bot, midlev, ktrop)."""
    nz = g.nz
    z = g.zsu
    kmid = _nearest(z, midlev)
    dudz = np.zeros(nz)
    for k in range(0, ktrop + 1):
        dudz[k] = bot + (top - bot) / (z[ktrop] - z[0]) * z[k]
    dudz[ktrop:] = top
    w = np.zeros(nz)
    for k in range(kmid + 1, nz):
        w[k] = w[k - 1] + dudz[k] * (z[k] - z[k - 1])
    for k in range(kmid - 1, -1, -1):
        w[k] = w[k + 1] - dudz[k] * (z[k + 1] - z[k])
    return w


def _mirror(s: np.ndarray) -> None:
    """mirror_boundaries (boundaries.cpp:363-379), levels 1..NZ-2."""
    s[0, :, 1:-1] = s[1, :, 1:-1]
    s[-1, :, 1:-1] = s[-2, :, 1:-1]
    s[:, 0, 1:-1] = s[:, 1, 1:-1]
    s[:, -1, 1:-1] = s[:, -2, 1:-1]


def _add_rotational_wind(g: _Grid, stream: np.ndarray, ub: np.ndarray, vb: np.ndarray) -> None:
    """u -= d(psi)/dy and v += d(psi)/dx by four-point averages
    (data_initializer.cpp:368-377), i, j interior, k < NZ-1."""
    S = stream
    ub[1:-1, 1:-1, :-1] += -0.25 * ((S[:-2, 2:, :-1] + S[1:-1, 2:, :-1]) - (S[:-2, :-2, :-1] + S[1:-1, :-2, :-1])) \
        * (1.0 / g.dy)
    vb[1:-1, 1:-1, :-1] += 0.25 * ((S[2:, :-2, :-1] + S[2:, 2:, :-1]) - (S[:-2, :-2, :-1] + S[:-2, 2:, :-1])) \
        * (1.0 / g.dx)


def _pressure_from_winds(g: _Grid, p: np.ndarray, u: np.ndarray) -> None:
    """get_pressure_from_winds: geostrophic integration in y, i < NX-1."""
    for j in range(1, g.ny):
        umid = 0.25 * (u[:-1, j - 1, :] + u[1:, j - 1, :] + u[:-1, j, :] + u[1:, j, :])
        p[:-1, j, :] = p[:-1, j - 1, :] - (umid * g.f[j] + 0.0) * g.dy


def _balanced_pass(g: _Grid, amp: float, ub, vb, pb, thb, tbv, pib, base_i, base_j):
    """One wind / pressure / theta pass of the ITCZ initialiser
    (data_initializer.cpp:362-406 and 488-534)."""
    stream = _streamfunction(g, _shear_zone(g, amp))
    _add_rotational_wind(g, stream, ub, vb)
    _mirror(ub)
    _pressure_from_winds(g, pb, ub)
    pb -= pb[base_i, base_j, :].copy()[None, None, :]
    _mirror(pb)
    z = g.zsu
    pb[:, :, 0] = pb[:, :, 1] - (z[1] - z[0]) * (pb[:, :, 2] - pb[:, :, 1]) / (z[2] - z[1])
    pb[:, :, -1] = pb[:, :, -2]
    thb[:, :, 1:] = tbv[None, None, 1:] * (pb[:, :, 1:] - pb[:, :, :-1]) / (GRAV * (z[1:] - z[:-1]))[None, None, :]
    pb[:] = pb / (CP * tbv)[None, None, :] + pib[None, None, :]


def itcz_shear_state(nx, ny, nz, dx, dz, corner_lat, corner_lon, hor_shear=1.0e-4, vert_shear0=-2.0e-3,
                     vert_shear1=-1.0e-3, ktrop=37) -> dict:
    """Basic state of initialize_basic_state_ITCZ_shear2(hor_shear,
    vert_shear0, vert_shear1) on a uniform grid, with ktrop clamped to
    NZ - 2.  Returns ubar, vbar, wbar, thbar, qbar, pbar [NX][NY][NZ] and the
    columns tb, qb (the sounding on the model levels)."""
    g = _Grid(nx, ny, nz, dx, dx, dz, corner_lat, corner_lon)
    ktrop = min(ktrop, nz - 2)
    tb, qb = sounding_20n_88e(g.zsu)
    tbv, pib, rhou, rhow = column_state(tb, qb, g.zsu)
    base_i, base_j = _nearest(g.lons, 88), _nearest(g.lats, 20)
    shape = (nx, ny, nz)
    ub, vb, wb = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    thb, qbb, pb = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    control = 1.0e-4
    ub[:] = (_shear_profile(g, vert_shear0, vert_shear1, 4000, ktrop) + 3)[None, None, :]
    _balanced_pass(g, control, ub, vb, pb, thb, tbv, pib, base_i, base_j)
    # relative humidity: the 20N/88E column's, lowered south of 15N and north of 26N
    lat_pt = lambda lat: _nearest(g.lats, lat)  # noqa: E731
    y_min, y_max, y_min2, y_max2, y_min3 = lat_pt(5), lat_pt(15), lat_pt(26), lat_pt(30), lat_pt(20)
    dec, dec2, dec3 = 0.1, 0.1, 0.0
    slope = dec / float(y_max - y_min)
    slope2 = dec2 / float(y_max2 - y_min2)
    slope3 = dec3 / float(y_min2 - y_min3)
    drop = np.zeros(ny + 1)  # one spare slot: the first loop reads drop[j + 1] at j = y_max
    for j in range(y_max, y_min, -1):
        drop[j] = drop[j + 1] + slope
    for j in range(y_min, -1, -1):
        drop[j] = dec
    for j in range(y_min3, y_min2):
        drop[j] = drop[j - 1] + slope3
    for j in range(y_min2, y_max2):
        drop[j] = drop[j - 1] + slope2
    for j in range(y_max2, ny):
        drop[j] = drop[j - 1]
    drop = drop[:ny]
    base_relh = qb / _qvsat(tb * pib, P0 * pib ** (CP / RD))
    temp = (thb[:, :, 1:-1] + tb[None, None, 1:-1]) * pb[:, :, 1:-1]
    pres = P0 * pb[:, :, 1:-1] ** (CP / RD)
    qbb[:, :, 1:-1] = (base_relh[None, None, 1:-1] - drop[None, :, None]) * _qvsat(temp, pres) - qb[None, None, 1:-1]
    # final vorticity
    _balanced_pass(g, hor_shear - control, ub, vb, pb, thb, tbv, pib, base_i, base_j)
    for s in (thb, qbb, ub, vb):
        s[:, :, 0] = s[:, :, 1]
        s[:, :, -1] = s[:, :, -2]
    # basic-state vertical velocity (init_basic_state_vertical_velocity), flat ground
    dzu = g.zsw[1:] - g.zsw[:-1]
    for k in range(2, nz - 1):
        wb[1:-1, 1:-1, k] = (rhow[k - 1] / rhow[k]) * wb[1:-1, 1:-1, k - 1] + (rhou[k - 1] / rhow[k]) * (
            -(ub[2:, 1:-1, k - 1] - ub[1:-1, 1:-1, k - 1]) / dx
            - (vb[1:-1, 2:, k - 1] - vb[1:-1, 1:-1, k - 1]) / g.dy) * dzu[k]
    wb[1:-1, 1:-1, nz - 1] = wb[1:-1, 1:-1, nz - 2]
    return {"ubar": ub, "vbar": vb, "wbar": wb, "thbar": thb, "qbar": qbb, "pbar": pb, "tb": tb, "qb": qb,
            "tbv": tbv, "pib": pib, "rhou": rhou, "rhow": rhow, "lats": g.lats, "lons": g.lons, "f": g.f,
            "base_ij": (base_i, base_j)}


# ---------------------------------------------------------------------------
# the vortex
# ---------------------------------------------------------------------------
def vortex(state: dict, nx, ny, nz, dx, dz, r_end, zm, zt, tmax, tmin, xpos, ypos):
    """Perturbation u, v, theta of initialize_vortex(r_end, zm, zt, tmax, tmin,
    ..., xpos, ypos) with no moisture anomaly: theta' = t_z(z) t_r(r), the
    hydrostatic geopotential of theta'/theta, the gradient wind of that
    geopotential, interpolated from radius to the grid (Cartesian winds at
    cell centres), then staggered onto the u and v points."""
    zsu = (np.arange(nz, dtype=np.float64) - 0.5) * dz
    tb = state["tb"]
    nr = int(r_end / dx)
    zmid = 0.5 * (zm + zt)
    t_z = np.where(zsu <= zm, tmin * np.exp(-(zsu * zsu) / (zm * zm / 8.0)),
                   tmax * np.exp(-((zsu - zmid) * (zsu - zmid)) / ((zt - zm) * (zt - zm) / 32.0)))
    r = np.arange(nr, dtype=np.float64)
    t_r = np.exp(-dx * r * dx * r / (r_end * r_end / 8.0))
    phi = np.zeros((nz, nr))
    for k in range(nz - 2, 0, -1):
        tmid = 0.5 * (t_z[k] * t_r + t_z[k + 1] * t_r) / ((tb[k] + tb[k + 1]) * 0.5) + 0.61 * 0.0
        phi[k] = phi[k + 1] - GRAV * tmid * (zsu[k + 1] - zsu[k])
    fcor = 2 * 7.292e-5 * np.sin(state["lats"][ypos] * TRIGPI / 180.0)
    vr = np.zeros((nz, nr))
    R = r[1:nr - 1] * dx
    grad = np.abs(phi[:, 2:] - phi[:, :-2])
    low = phi[:, 1:nr - 1] < 0
    v_low = -0.5 * fcor * R + 0.5 * np.sqrt(fcor * fcor * R * R + 4 * R * 0.5 * grad * (1.0 / dx))
    rad = np.maximum(fcor * fcor * R * R - 4 * R * 0.5 * grad * (1.0 / dx), 0.0)
    v_high = -(0.5 * fcor * R - 0.5 * np.sqrt(rad))
    vr[:, 1:nr - 1] = np.where(low, v_low, v_high)
    u = np.zeros((nx, ny, nz))
    v = np.zeros((nx, ny, nz))
    th = np.zeros((nx, ny, nz))
    for i in range(max(xpos - nr, 1), min(xpos + nr, nx)):
        for j in range(max(ypos - nr, 1), min(ypos + nr, ny)):
            di, dj = float(i - xpos), float(j - ypos)
            dist = np.sqrt(di * di + dj * dj)
            ind = int(dist)
            frac = dist - float(ind)
            if ind >= nr - 2:
                continue
            th[i, j, 1:] += t_z[1:] * ((1.0 - frac) * t_r[ind] + frac * t_r[ind + 1])
            if ind != 0:
                iproj = abs(dj) / (float(ind) + frac)
                jproj = abs(di) / (float(ind) + frac)
                wm = (1.0 - frac) * vr[1:, ind] + frac * vr[1:, ind + 1]
                u[i, j, 1:] += wm * iproj if j < ypos else -wm * iproj
                v[i, j, 1:] += -wm * jproj if i < xpos else wm * jproj
    us = np.zeros_like(u)
    us[1:, 1:, :] = 0.5 * (u[1:, 1:, :] + u[:-1, 1:, :])
    vs = np.zeros_like(v)
    vs[1:, 1:, :] = 0.5 * (v[1:, :-1, :] + v[1:, 1:, :])
    return us, vs, th
