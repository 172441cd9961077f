"""CPU oracle for the VlaPy time step -- TEST INFRASTRUCTURE ONLY.

This module restates, in NumPy/SciPy, the arithmetic of the reference VlaPy
time step (joglekara/VlaPy).  It is what the CUDA path is tested against: only the
test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it.  The product package ``vlapy_gb300`` never calls
into it and has no CPU fallback.

Every function cites the reference file:line whose arithmetic it follows.  The
operation order matches the reference's NumPy expressions (same ufuncs, same
``scipy.fft`` calls, same ``np.trapezoid`` reductions) so that, on the same
inputs and the same NumPy/SciPy build, oracle and reference agree bit for bit;
``tests/golden`` holds fixtures produced by the reference itself that pin this.

The reference itself is vectorised NumPy with one Python-level loop (the
tridiagonal sweep over v); the oracle keeps that structure so its timing is a
faithful stand-in for the reference CPU path.

Third-party arithmetic used by the reference and therefore here:
  * scipy.fft.fft / ifft (pocketfft, as shipped in SciPy; unpinned by the
    reference's setup.py:25-35),
  * numpy.trapezoid (numpy >= 2 name of numpy.trapz),
  * scipy.special.wofz + scipy.optimize.newton (dispersion root),
  * scipy.interpolate.RectBivariateSpline and interp1d (the semi-Lagrangian
    steppers; FITPACK inside SciPy).
"""

from __future__ import annotations

import math

import numpy as np
from scipy import fft as sfft
from scipy import interpolate, optimize, special


def trapz(y, dx, axis=-1):
    """np.trapz with constant spacing (the reference calls np.trapz everywhere,
    e.g. vlapy/core/field.py:36; NumPy 2 renamed it trapezoid)."""
    return np.trapezoid(y, dx=dx, axis=axis)


# --------------------------------------------------------------------------
# grids and initial state -- vlapy/initializers.py
# --------------------------------------------------------------------------

def velocity_axis(vmax, nv):
    """dv, cell-centred v and kv = 2*pi*fftfreq(nv, dv).
    Follows vlapy/initializers.py:56-69."""
    dv = 2 * vmax / nv
    v = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    kv = np.fft.fftfreq(v.size, d=dv) * 2.0 * np.pi
    return dv, v, kv


def spatial_axis(xmin, xmax, nx):
    """dx, cell-centred x, kx and 1/kx with the k=0 entry set to zero.
    Follows vlapy/initializers.py:72-89."""
    dx = (xmax - xmin) / nx
    x = np.linspace(xmin + dx / 2.0, xmax - dx / 2.0, nx)
    kx = np.fft.fftfreq(x.size, d=dx) * 2.0 * np.pi
    inv_kx = np.zeros_like(kx)
    inv_kx[1:] = 1.0 / kx[1:]
    return dx, x, kx, inv_kx


def maxwellian(nx, nv, vmax=6.0):
    """Unit-temperature Maxwellian normalised to unit density by trapz, one
    identical row per x.  Follows vlapy/initializers.py:29-53."""
    dv = 2.0 * vmax / nv
    v = np.linspace(-vmax + dv / 2.0, vmax - dv / 2.0, nv)
    f = np.zeros([nx, nv], dtype=np.float64)
    row = np.exp(-(v ** 2.0) / 2.0)
    f[:] = row[None, :]
    return f / trapz(f, dx=dv, axis=1)[:, None]


def shifted_maxwellian(nx, v, v0, vshift):
    """Drifting Maxwellian used by the collision tests (tests/helpers.py:26-34)."""
    dv = v[2] - v[1]
    f = np.zeros((nx, v.size))
    f[:] = np.exp(-((v - vshift) ** 2.0) / 2.0 / v0)
    return f / (trapz(f, dx=dv, axis=1)[:, None])


# --------------------------------------------------------------------------
# advection -- vlapy/core/vlasov.py
# --------------------------------------------------------------------------

def vdfdx_exponential(f, kx, v, dt):
    """x-advection by the exponential integrator: Re IFFT_x(exp(-i kx v dt) FFT_x f).
    Follows vlapy/core/vlasov.py:83-110 (expression at :106-108)."""
    # written as one expression: NumPy elides the temporary phase array into an
    # in-place multiply whose rounding can differ in the last bit from a
    # multiply by a named array, and the reference uses the inline form
    return np.real(sfft.ifft(np.exp(-1j * kx[:, None] * dt * v) * sfft.fft(f, axis=0), axis=0))


def edfdv_exponential(f, e, kv, dt):
    """v-advection by the exponential integrator: Re IFFT_v(exp(-i kv E dt) FFT_v f).
    Follows vlapy/core/vlasov.py:113-140 (expression at :136-138)."""
    return np.real(sfft.ifft(np.exp(-1j * kv * dt * e[:, None]) * sfft.fft(f, axis=1), axis=1))


def edfdv_center_differenced(f, e, dv, dt):
    """Second-order centred E df/dv update (vlapy/core/vlasov.py:143-165)."""
    return f - e[:, None] * np.gradient(f, dv, axis=1, edge_order=2) * dt


def padded_axis(ax):
    """The axis with one node of spacing ax[2] - ax[1] added at each end
    (vlapy/core/vlasov.py:27-39)."""
    out = np.zeros(ax.size + 2)
    out[1:-1] = ax
    out[0] = ax[0] - (ax[2] - ax[1])
    out[-1] = ax[-1] + (ax[2] - ax[1])
    return out


def vdfdx_sl(f, x, v, dt):
    """Backward semi-Lagrangian x step (vlapy/core/vlasov.py:42-80): the s = 0
    bicubic spline (scipy RectBivariateSpline, FITPACK) of f over the x axis
    extended by one periodic row at each end, evaluated at (x - v dt, v)."""
    xm, vm = np.meshgrid(x, v, indexing="ij")
    f_pad = np.zeros((x.size + 2, v.size))
    f_pad[1:-1, :] = f
    f_pad[0, :] = f[-1, :]
    f_pad[-1, :] = f[0, :]
    spline = interpolate.RectBivariateSpline(padded_axis(x), v, f_pad)
    return spline(xm.flatten() - vm.flatten() * dt, vm.flatten(), grid=False).reshape((x.size, v.size))


def edfdv_sl(f, e, x, v, dt):
    """Backward semi-Lagrangian v step (vlapy/core/vlasov.py:168-210): the
    bicubic spline over the v axis extended by one periodic column at each
    end, evaluated at (x, v - e(x) dt), with e taken through a cubic
    interp1d at the grid nodes as the reference does."""
    xm, vm = np.meshgrid(x, v, indexing="ij")
    xm = xm.flatten()
    vm = vm.flatten()
    f_pad = np.zeros((x.size, v.size + 2))
    f_pad[:, 1:-1] = f
    f_pad[:, 0] = f[:, -1]
    f_pad[:, -1] = f[:, 0]
    em = interpolate.interp1d(x, e, kind="cubic")(xm)
    spline = interpolate.RectBivariateSpline(x, padded_axis(v), f_pad)
    return spline(xm, vm - em * dt, grid=False).reshape((x.size, v.size))


# --------------------------------------------------------------------------
# field solve -- vlapy/core/field.py
# --------------------------------------------------------------------------

def charge_density(f, dv):
    """n(x) = trapz_v f (vlapy/core/field.py:27-36)."""
    return trapz(f, dx=dv, axis=1)


def spectral_poisson(net_charge, inv_kx):
    """E = Re IFFT(i * (1/kx) * FFT(rho)) (vlapy/core/field.py:39-49)."""
    return np.real(sfft.ifft(1j * inv_kx * sfft.fft(net_charge)))


def field_from_density(n, inv_kx):
    """Field of the electrons against a unit ion background
    (vlapy/core/field.py:52-63)."""
    return spectral_poisson(1.0 - n, inv_kx)


def total_field(driver, f, dv, inv_kx):
    """driver + self-consistent field (vlapy/core/field.py:66-88)."""
    return driver + field_from_density(charge_density(f, dv), inv_kx)


# --------------------------------------------------------------------------
# collisions -- vlapy/core/collisions.py
# --------------------------------------------------------------------------

def lenard_bernstein_diagonals(f, v, nu, dt, dv):
    """Tridiagonal (a, b, c) of the implicit Lenard-Bernstein operator.
    Follows vlapy/core/collisions.py:26-83."""
    nx, nv = f.shape
    vth2 = trapz(f * v[None, :] ** 2.0, dx=dv, axis=1)
    a = nu * dt * np.ones((nx, nv - 1)) * (-vth2[:, None] / dv ** 2.0 + v[None, :-1] / 2 / dv)
    b = 1.0 + nu * dt * np.ones((nx, nv)) * (2 * vth2[:, None] / dv ** 2.0)
    c = nu * dt * np.ones((nx, nv - 1)) * (-vth2[:, None] / dv ** 2.0 - v[None, 1:] / 2 / dv)
    return a, b, c


def dougherty_diagonals(f, v, nu, dt, dv):
    """Tridiagonal (a, b, c) of the implicit Dougherty operator; the drift and
    temperature moments are plain trapz integrals, not divided by density.
    Follows vlapy/core/collisions.py:86-160."""
    nx, nv = f.shape
    ubar = trapz(f * v[None, :], dx=dv, axis=1)
    vth2 = trapz(f * (v[None, :] - ubar[:, None]) ** 2.0, dx=dv, axis=1)
    a = nu * dt * np.ones((nx, nv - 1)) * (
        -vth2[:, None] / dv ** 2.0 + (v[None, :-1] - ubar[:, None]) / 2.0 / dv)
    b = 1.0 + nu * dt * np.ones((nx, nv)) * (2.0 * vth2[:, None] / dv ** 2.0)
    c = nu * dt * np.ones((nx, nv - 1)) * (
        -vth2[:, None] / dv ** 2.0 - (v[None, 1:] - ubar[:, None]) / 2.0 / dv)
    return a, b, c


def thomas_batched(a, b, c, d):
    """Thomas algorithm, vectorised over x and looping over v; A[j, j-1] = a[j-1],
    A[j, j] = b[j], A[j, j+1] = c[j].  Follows vlapy/core/collisions.py:222-265."""
    nv = b.shape[1]
    bb = b.copy()
    cc = c.copy()
    aa = a.copy()
    dd = d.copy()
    for j in range(1, nv):
        m = aa[:, j - 1] / bb[:, j - 1]
        bb[:, j] = bb[:, j] - m * cc[:, j - 1]
        dd[:, j] = dd[:, j] - m * dd[:, j - 1]
    x = bb
    x[:, -1] = dd[:, -1] / bb[:, -1]
    for j in range(nv - 2, -1, -1):
        x[:, j] = (dd[:, j] - cc[:, j] * x[:, j + 1]) / bb[:, j]
    return x


def dense_solve_rows(a, b, c, f):
    """Per-x dense solve (vlapy/core/collisions.py:163-219); cross-check only."""
    out = f.copy()
    for ix in range(f.shape[0]):
        m = np.diag(a[ix], -1) + np.diag(b[ix], 0) + np.diag(c[ix], 1)
        out[ix] = np.linalg.solve(m, f[ix])
    return out


def collision_step(f, v, nu, dt, dv, operator="dg"):
    """Implicit Fokker-Planck step: identity when nu == 0, else build the
    diagonals and solve.  Follows vlapy/core/step.py:70-113."""
    if nu == 0.0:
        return f
    if operator == "dg":
        a, b, c = dougherty_diagonals(f, v, nu, dt, dv)
    elif operator == "lb":
        a, b, c = lenard_bernstein_diagonals(f, v, nu, dt, dv)
    else:
        raise NotImplementedError(operator)
    return thomas_batched(a, b, c, f)


# --------------------------------------------------------------------------
# driver -- vlapy/field_driver.py
# --------------------------------------------------------------------------

def driver_tanh(x, pulses, t):
    """Sum over pulses of 0.5*(tanh((t-tL)/twL) - tanh((t-tR)/twR)) * k * a0 *
    sin(k x - w t).  Follows vlapy/field_driver.py:24-50."""
    total = np.zeros(x.size)
    for p in pulses.values():
        k, w = p["k0"], p["w0"]
        env = 0.5 * (np.tanh((t - p["t_L"]) / p["t_wL"]) - np.tanh((t - p["t_R"]) / p["t_wR"]))
        total += env * k * p["a0"] * np.sin(k * x - w * t)
    return total


def driver_sin2(x, k, w, a0, t_end, t):
    """a0 * sin(k x - w t) * sin^2(pi t / t_end) for t in [0, t_end], zero after:
    the driven-wave workload's envelope (not in the reference; the reference
    step accepts any driver closure, vlapy/core/vlasov_poisson.py:55)."""
    if t < 0.0 or t > t_end:
        return np.zeros(x.size)
    s = math.sin(math.pi * t / t_end)
    return (a0 * (s * s)) * np.sin(k * x - w * t)


# --------------------------------------------------------------------------
# time integrators -- vlapy/core/vlasov_poisson.py
# --------------------------------------------------------------------------

class Operators:
    """Bundle of the sub-operator closures a VP integrator composes
    (vlapy/core/step.py:29-67)."""

    def __init__(self, x, v, kx, kv, inv_kx, dv, driver=None, vdfdx="exponential", edfdv="exponential"):
        self.x, self.v, self.kx, self.kv, self.inv_kx, self.dv = x, v, kx, kv, inv_kx, dv
        self.driver = driver if driver is not None else (lambda t: np.zeros(x.size))
        # the stepper names of vlapy/core/vlasov.py:213-260
        if vdfdx not in ("exponential", "sl") or edfdv not in ("exponential", "cd2", "sl"):
            raise NotImplementedError((vdfdx, edfdv))
        self.vdfdx_name, self.edfdv_name = vdfdx, edfdv

    def vdfdx(self, f, dt):
        if self.vdfdx_name == "sl":
            return vdfdx_sl(f, self.x, self.v, dt)
        return vdfdx_exponential(f, self.kx, self.v, dt)

    def edfdv(self, f, e, dt):
        if self.edfdv_name == "sl":
            return edfdv_sl(f, e, self.x, self.v, dt)
        if self.edfdv_name == "cd2":
            return edfdv_center_differenced(f, e, self.dv, dt)
        return edfdv_exponential(f, e, self.kv, dt)

    def field(self, t, f):
        return total_field(self.driver(t), f, self.dv, self.inv_kx)


def leapfrog(ops, e, f, t, dt):
    """Strang split: half kick, drift, field solve at t+dt, half kick.
    Follows vlapy/core/vlasov_poisson.py:24-60."""
    f = ops.edfdv(f, e, 0.5 * dt)
    f = ops.vdfdx(f, dt)
    e = ops.field(t + dt, f)
    f = ops.edfdv(f, e, 0.5 * dt)
    return e, f


PEFRL_XSI = 0.1786178958448091
PEFRL_LAMBDA = -0.2123418310626054
PEFRL_CHI = -0.6626458266981849e-1


def pefrl(ops, e, f, t, dt):
    """Fourth-order PEFRL splitting (Omelyan, Mryglod & Folk 2002).
    Follows vlapy/core/vlasov_poisson.py:63-154."""
    d1 = PEFRL_XSI * dt
    d2 = PEFRL_CHI * dt
    d3 = (1.0 - 2.0 * (PEFRL_CHI + PEFRL_XSI)) * dt
    d4, d5 = d2, d1
    k1 = 0.5 * (1.0 - 2.0 * PEFRL_LAMBDA) * dt
    k2 = PEFRL_LAMBDA * dt
    k3, k4 = k2, k1
    f = ops.vdfdx(f, d1)
    e = ops.field(t + d1, f)
    f = ops.edfdv(f, e, k1)
    f = ops.vdfdx(f, d2)
    e = ops.field(t + d1 + d2, f)
    f = ops.edfdv(f, e, k2)
    f = ops.vdfdx(f, d3)
    e = ops.field(t + d1 + d2 + d3, f)
    f = ops.edfdv(f, e, k3)
    f = ops.vdfdx(f, d4)
    e = ops.field(t + d1 + d2 + d3 + d4, f)
    f = ops.edfdv(f, e, k4)
    f = ops.vdfdx(f, d5)
    e = ops.field(t + d1 + d2 + d3 + d4 + d5, f)
    return e, f


H6 = dict(
    a1=0.168735950563437422448196, a2=0.377851589220928303880766,
    a3=-0.093175079568731452657924, b1=0.049086460976116245491441,
    b2=0.264177609888976700200146, b3=0.186735929134907054308413,
    c1=-0.000069728715055305084099, c2=-0.000625704827430047189169,
    c3=-0.002213085124045325561636, d2=-2.916600457689847816445691e-6,
    d3=3.048480261700038788680723e-5, e3=4.985549387875068121593988e-7,
)


def sixth_order(ops, e, f, t, dt):
    """Sixth-order Hamiltonian splitting (Casas, Crouseilles, Faou &
    Mehrenberger 2017).  Follows vlapy/core/vlasov_poisson.py:157-232,
    including its field-solve times t + a_i*dt."""
    h = H6
    D1 = h["b1"] + 2.0 * h["c1"] * dt ** 2.0
    D2 = h["b2"] + 2.0 * h["c2"] * dt ** 2.0 + 4.0 * h["d2"] * dt ** 4.0
    D3 = (h["b3"] + 2.0 * h["c3"] * dt ** 2.0 + 4.0 * h["d3"] * dt ** 4.0
          - 8.0 * h["e3"] * dt ** 6.0)
    a1, a2, a3 = h["a1"], h["a2"], h["a3"]
    f = ops.edfdv(f, e, D1 * dt)
    for a, D in ((a1, D2), (a2, D3), (a3, D3), (a2, D2), (a1, D1)):
        f = ops.vdfdx(f, a * dt)
        e = ops.field(t + a * dt, f)
        f = ops.edfdv(f, e, D * dt)
    return e, f


INTEGRATORS = {"leapfrog": leapfrog, "pefrl": pefrl, "h-sixth": sixth_order}


# --------------------------------------------------------------------------
# storage step -- vlapy/core/step.py:116-283 and vlapy/outer_loop.py:149-245
# --------------------------------------------------------------------------

FIELD_KEYS = ("e", "driver", "n", "j", "T", "q", "fv4", "vN")
SERIES_KEYS = ("mean_n", "mean_j", "mean_T", "mean_e2", "mean_de2", "mean_f2", "mean_flogf")


def new_storage(f, e, nt, n_modes=None):
    """Inner-loop storage dict (vlapy/outer_loop.py:149-215).  n_modes=None
    stores all of f; otherwise the first n_modes x-Fourier modes as complex64."""
    nx, nv = f.shape
    if n_modes is None:
        stored = np.zeros((nt, nx, nv), dtype=np.float64)
        stored[0] = f
    else:
        stored = np.zeros((nt, n_modes, nv), dtype=np.complex64)
        stored[0] = np.fft.fft(f, axis=0)[:n_modes]
    return {
        "time_batch": np.zeros(nt),
        "e": np.array(e),
        "f": np.array(f),
        "stored_f": stored,
        "mean_cum_de2_previous": 0.0,
        "series": {k: np.zeros(nt) for k in SERIES_KEYS},
        "fields": {k: np.zeros((nt, nx)) for k in FIELD_KEYS},
    }


def store(st, e, de, f, i, v, dv, n_modes=None):
    """Per-step storage: stored_f, the six velocity moments, e and the driver,
    then the x-means.  Follows vlapy/core/step.py:116-283."""
    if n_modes is None:
        st["stored_f"][i] = f
    else:
        st["stored_f"][i] = sfft.fft(f, axis=0)[:n_modes]
    st["e"], st["f"] = e, f
    fl = st["fields"]
    fl["e"][i] = e
    fl["driver"][i] = de
    fl["n"][i] = trapz(f, dx=dv, axis=1)
    fl["j"][i] = trapz(f * v, dx=dv, axis=1)
    fl["T"][i] = trapz(f * v ** 2, dx=dv, axis=1)
    fl["q"][i] = trapz(f * v ** 3, dx=dv, axis=1)
    fl["fv4"][i] = trapz(f * v ** 4, dx=dv, axis=1)
    fl["vN"][i] = trapz(f * v ** 5, dx=dv, axis=1)
    se = st["series"]
    se["mean_n"][i] = np.mean(fl["n"][i], axis=0)
    se["mean_j"][i] = np.mean(fl["j"][i], axis=0)
    se["mean_T"][i] = np.mean(fl["T"][i], axis=0)
    se["mean_e2"][i] = np.mean(e ** 2.0, axis=0)
    se["mean_de2"][i] = np.mean(de ** 2.0, axis=0)
    se["mean_f2"][i] = np.mean(trapz(np.real(f) ** 2.0, dx=dv, axis=1), axis=0)
    with np.errstate(invalid="ignore", divide="ignore"):
        se["mean_flogf"][i] = np.mean(trapz(f * np.log(f), dx=dv, axis=1), axis=0)
    return st


def post_inner_loop(st):
    """Cumulative driver energy and the two energy-balance series
    (vlapy/outer_loop.py:218-245)."""
    se = st["series"]
    se["mean_cum_de2"] = st["mean_cum_de2_previous"] + np.cumsum(se["mean_de2"])
    se["mean_t_plus_e2_minus_cum_de2"] = se["mean_T"] + (se["mean_e2"] - se["mean_cum_de2"])
    se["mean_t_plus_e2_plus_cum_de2"] = se["mean_T"] + se["mean_e2"] + se["mean_de2"]
    st["mean_cum_de2_previous"] = se["mean_cum_de2"][-1]
    return st


class OracleRun:
    """One VlaPy run held on the host: VP step, FP step and storage step in the
    order of vlapy/core/step.py:286-328, driven like vlapy/outer_loop.py:248-281."""

    def __init__(self, nx, nv, xmax, vmax, dt, nu=0.0, operator="dg",
                 integrator="leapfrog", driver=None, xmin=0.0, n_modes=None, vdfdx="exponential",
                 edfdv="exponential"):
        self.dx, self.x, self.kx, self.inv_kx = spatial_axis(xmin, xmax, nx)
        self.dv, self.v, self.kv = velocity_axis(vmax, nv)
        self.dt, self.nu, self.operator = dt, nu, operator
        self.ops = Operators(self.x, self.v, self.kx, self.kv, self.inv_kx, self.dv, driver, vdfdx, edfdv)
        self.vp = INTEGRATORS[integrator]
        self.n_modes = n_modes

    def step(self, e, f, t):
        e, f = self.vp(self.ops, e, f, t, self.dt)
        f = collision_step(f, self.v, self.nu, self.dt, self.dv, self.operator)
        return e, f

    def timestep(self, st, i):
        """vlapy/core/step.py:302-326."""
        t = st["time_batch"][i]
        de = st["driver_array_batch"][i]
        e, f = self.step(st["e"], st["f"], t)
        store(st, e, de, f, i, self.v, self.dv, self.n_modes)
        return st, i

    def inner_loop(self, time_array, driver_array, st):
        """vlapy/outer_loop.py:265-272."""
        st["time_batch"] = time_array
        st["driver_array_batch"] = driver_array
        for it in range(time_array.size):
            st, _ = self.timestep(st, it)
        return post_inner_loop(st)


# --------------------------------------------------------------------------
# dispersion root and damping fit -- vlapy/diagnostics/z_function.py
# --------------------------------------------------------------------------

def plasma_z(zeta):
    """Z(zeta) = i sqrt(pi) w(zeta) (vlapy/diagnostics/z_function.py:6-13)."""
    return 1j * math.sqrt(math.pi) * special.wofz(zeta)


def epw_root(k0, wp=1.0, vth=1.0):
    """Complex frequency of the electron plasma wave: Newton root of
    1 - chi Z'(zeta) with Z' = -2(1 + zeta Z), chi = (wp/(vth k))^2/2.
    Follows vlapy/diagnostics/z_function.py:26-50."""
    guess = np.sqrt(wp ** 2.0 + 3 * (k0 * vth) ** 2.0)
    chi = np.power(wp / (vth * k0), 2.0) / 2.0

    def eps(z):
        return 1.0 - chi * (-2.0 * (1.0 + z * plasma_z(z)))

    root = optimize.newton(eps, guess)
    return root * k0 * vth * np.sqrt(2.0)


def mode_amplitude(e_hist, mode=1):
    """|FFT_x(E)[mode]| per stored step (vlapy/diagnostics/low_level_helpers.py:84)."""
    return np.abs(np.fft.fft(e_hist, axis=1)[:, mode])


def envelope_fit(t, amp, t_min=None, t_max=None):
    """Damping rate and frequency from the peaks of |E_k|(t): a least-squares
    line through log(peak heights) gives the rate, twice the mean peak spacing
    gives the period of Re(E_k).  The reference estimator
    (vlapy/diagnostics/low_level_helpers.py:69-87) averages d log|E_k|/dt and
    is biased for undriven runs, so both the CPU oracle and the GPU runs are
    measured with this one fit."""
    sel = np.ones_like(t, dtype=bool)
    if t_min is not None:
        sel &= t >= t_min
    if t_max is not None:
        sel &= t <= t_max
    tt, aa = t[sel], amp[sel]
    pk = np.where((aa[1:-1] > aa[:-2]) & (aa[1:-1] >= aa[2:]))[0] + 1
    if pk.size < 3:
        return float("nan"), float("nan")
    # parabolic refinement of each peak in log space
    tp, lp = [], []
    h = tt[1] - tt[0]
    for p in pk:
        y0, y1, y2 = np.log(aa[p - 1]), np.log(aa[p]), np.log(aa[p + 1])
        den = y0 - 2 * y1 + y2
        off = 0.5 * (y0 - y2) / den if den != 0 else 0.0
        tp.append(tt[p] + off * h)
        lp.append(y1 - 0.25 * (y0 - y2) * off)
    tp, lp = np.array(tp), np.array(lp)
    rate = np.polyfit(tp, lp, 1)[0]
    # |E_k1| peaks twice per oscillation period of the standing wave
    freq = np.pi / np.mean(np.diff(tp))
    return float(rate), float(freq)
