"""CPU oracle for the microscope stage after the backend: objective focalisation and the
incoherent spectrum sum. TEST INFRASTRUCTURE ONLY — it checks the CUDA path and is never
called by the product.

Restates, in numpy FP64:
  * OpticalFields wavevector grid   HighLevelPythonInterface/nemaktis/light_propagator.py:576-596
  * objective filter and NA mask    light_propagator.py:614-646, update_NA_objective :702-705
  * focus_fields                    light_propagator.py:708-719
  * Jones matrices                  nemaktis/field_viewer.py:472-513
  * _update_specter                 field_viewer.py:348-388
  * _update_averaged_specter        field_viewer.py:391-455 (q_int_func, get_q_idx :515-518)

Pinned against the reference itself: tests/golden/make_golden.py runs the reference's own
OpticalFields/FieldViewer code and the CPU tests compare this module with its output.
"""
import numpy as np

WAVEPLATES = ("No", "Quarter-wave", "Half-wave", "Tint-sensitive")


def wavevectors(max_NA_condenser, Nr, koehler_1D=False, dims=(2, 2)):
    """Illumination wavevectors (Nq, 2): a 1-D line of 2Nr-1 points when the mesh is 1-D and
    Koehler 1-D is asked for, else 1 + 3Nr(Nr-1) points on hexagonal rings (:576-596)."""
    Nr = int(Nr)
    if koehler_1D and (dims[0] == 1 or dims[1] == 1):
        axis = 1 if dims[0] == 1 else 0
        q = np.zeros((2 * Nr - 1, 2))
        for ir in range(1, Nr):
            b = ir * max_NA_condenser / (Nr - 1)
            q[Nr - 1 + ir, axis] = b
            q[Nr - 1 - ir, axis] = -b
        return q
    q = np.zeros((1 + 3 * Nr * (Nr - 1), 2))
    for ir in range(1, Nr):
        b = ir * max_NA_condenser / (Nr - 1)
        for k in range(6 * ir):
            phi = k * np.pi / (3 * ir)
            q[1 + 3 * ir * (ir - 1) + k] = (b * np.cos(phi), b * np.sin(phi))
    return q


def spacing(length, n):
    """Mesh spacing length/max(1, n-1) (:599)."""
    return length / max(1.0, float(n) - 1.0)


def _kgrid(n, d):
    """Centred FFT frequencies ((i + n/2) mod n - n/2) * 2pi / (n d) (:622-623)."""
    i = np.arange(n, dtype=np.float64)
    return np.fmod(i + 0.5 * n, n) - 0.5 * n


def objective_tables(wavelengths, n_out, q, Nx, Ny, dx, dy):
    """|k+p|^2, k0 and the objective filter exp(i(sqrt(kn^2-|k+p|^2) - kn)) (zero outside kn),
    each of shape (Nl, Nq, Ny, Nx) (:621-642)."""
    wl = np.asarray(wavelengths, np.float64)
    nout = np.broadcast_to(np.asarray(n_out, np.float64), wl.shape)
    kx = _kgrid(Nx, dx) * 2 * np.pi / (Nx * dx)
    ky = _kgrid(Ny, dy) * 2 * np.pi / (Ny * dy)
    k0 = (2 * np.pi / wl)[:, None, None, None]
    kn = (2 * np.pi * nout / wl)[:, None, None, None]
    px = k0 * q[None, :, 0, None, None]
    py = k0 * q[None, :, 1, None, None]
    ksq = (kx[None, None, None, :] + px) ** 2 + (ky[None, None, :, None] + py) ** 2
    kn_full = np.broadcast_to(kn, ksq.shape)
    inside = ksq < kn_full ** 2
    filt = np.zeros(ksq.shape, np.complex128)
    filt[inside] = np.exp(1j * (np.sqrt(kn_full[inside] ** 2 - ksq[inside]) - kn_full[inside]))
    return ksq, np.broadcast_to(k0, ksq.shape), filt


def focus_fields(vals, wavelengths, n_out, q, Nx, Ny, dx, dy, NA, zfoc_NA_corr, z):
    """focused = iFFT2( FFT2(vals) * F ), F = mask * filter^|zf| (conjugated when zf < 0),
    zf = z + NA^2 * zfoc_NA_corr, mask = |k+p|^2 < (k0 NA)^2 (:702-719). The power is the
    principal-branch complex power of numpy (exp(|zf| * Log filter), 0^0 = 1)."""
    ksq, k0, filt = objective_tables(wavelengths, n_out, q, Nx, Ny, dx, dy)
    mask = (ksq < (k0 * NA) ** 2).astype(np.float64)
    zf = z + NA ** 2 * zfoc_NA_corr
    a = abs(zf)
    if a == 0:
        p = np.ones_like(filt)
    else:
        p = np.zeros_like(filt)
        nz = filt != 0
        p[nz] = np.exp(a * np.log(filt[nz]))
    F = mask * p
    if zf < 0:
        F = np.conj(F)
    spec = np.fft.fft2(vals, axes=(3, 4))
    spec *= F[:, :, None, :, :]
    return np.fft.ifft2(spec, axes=(3, 4))


def _rot(angle):
    a = angle * np.pi / 180
    return np.cos(a), np.sin(a)


def polariser(angle):
    c, s = _rot(angle)
    return np.array([[c * c, c * s], [c * s, s * s]], np.complex128)


def waveplate(kind, angle, wavelength):
    """Jones matrix of a waveplate (:479-509); the tint-sensitive plate is a full wave at
    0.540 um and depends on the wavelength."""
    c, s = _rot(angle)
    if kind == "Quarter-wave":
        return np.exp(-1j * np.pi / 4) * np.array(
            [[c * c + 1j * s * s, (1 - 1j) * c * s], [(1 - 1j) * c * s, s * s + 1j * c * c]])
    if kind == "Half-wave":
        return np.exp(-1j * np.pi / 2) * np.array([[c * c - s * s, 2 * c * s], [2 * c * s, s * s - c * c]])
    if kind == "Tint-sensitive":
        g = np.exp(1j * np.pi * 0.540 / wavelength)
        gc = np.conj(g)
        return np.array([[gc * c * c + g * s * s, (gc - g) * c * s], [(gc - g) * c * s, gc * s * s + g * c * c]])
    raise ValueError("unknown waveplate " + repr(kind))


def optics_matrices(wavelengths, pol=False, pol_angle=0.0, ana=False, ana_angle=0.0,
                    lower="No", lower_angle=0.0, upper="No", upper_angle=0.0):
    """Per-wavelength matrices applied before (lower waveplate . polariser) and after
    (analyser . upper waveplate) the sample's Jones matrix (:360-384). Shapes (Nl, 2, 2)."""
    Nl = len(wavelengths)
    pre = np.tile(np.eye(2, dtype=np.complex128), (Nl, 1, 1))
    post = pre.copy()
    for l, wl in enumerate(wavelengths):
        m = np.eye(2, dtype=np.complex128)
        if pol:
            m = polariser(pol_angle)
        if lower != "No":
            m = waveplate(lower, lower_angle, wl) @ m
        pre[l] = m
        m = np.eye(2, dtype=np.complex128)
        if upper != "No":
            m = waveplate(upper, upper_angle, wl) @ m
        if ana:
            m = polariser(ana_angle) @ m
        post[l] = m
    return pre, post


def q_int_func(q, qp):
    """Primitive of the Koehler weight g(q) = q/(1-q^2) used by the integration rule (:515-516)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return q - np.arctanh(q) - qp * np.log(1 - q * q) / 2


def get_q_idx(r):
    """First wavevector index of ring r (:517-518)."""
    return 1 + 3 * r * (r - 1)


def koehler_weights(NA_condenser, max_NA_condenser, Nr, koehler_1D=False):
    """(q_start, weights): the spectrum is sum_k weights[k] * specter[q_start + k]
    (:391-455; the 2/NA^2 or 1/(2NA) factor is folded into the weights)."""
    if NA_condenser < 1e-8:
        return (Nr - 1 if koehler_1D else 0), np.ones(1)
    dq = max_NA_condenser / (Nr - 1) if (Nr > 1 and max_NA_condenser > 0) else 1.0
    rmax = min(Nr - 1, int(np.ceil(NA_condenser / dq)))
    na = NA_condenser
    if not koehler_1D:
        w = np.zeros(get_q_idx(rmax + 1))

        def put(a, b, v):  # python slice semantics of the reference's assignments
            w[a:b] = v
        if rmax == 1:
            w[0] = (q_int_func(na, dq) - q_int_func(0, dq)) / dq
            put(1, 7, (q_int_func(0, 0) - q_int_func(na, 0)) / (6 * dq))
        else:
            w[0] = (q_int_func(dq, dq) - q_int_func(0, dq)) / dq
            for r in range(1, rmax - 1):
                put(get_q_idx(r), get_q_idx(r + 1),
                    (q_int_func((r + 1) * dq, (r + 1) * dq) + q_int_func((r - 1) * dq, (r - 1) * dq)
                     - 2 * q_int_func(r * dq, r * dq)) / (6 * r * dq))
            with np.errstate(divide="ignore", invalid="ignore"):
                put(get_q_idx(rmax - 1), get_q_idx(rmax),
                    (q_int_func(na, rmax * dq) + q_int_func((rmax - 2) * dq, (rmax - 2) * dq)
                     - 2 * q_int_func((rmax - 1) * dq, (rmax - 1) * dq)) / (6 * (rmax - 1) * dq))
                put(get_q_idx(rmax), get_q_idx(rmax + 1),
                    (q_int_func((rmax - 1) * dq, (rmax - 1) * dq) - q_int_func(na, (rmax - 1) * dq))
                    / (6 * rmax * dq))
        return 0, w * (2 / na ** 2)
    edge = na - (rmax - 1) * dq
    w = np.full(2 * rmax + 1, dq)
    w[0] = w[-1] = edge ** 2 / (2 * dq)
    if rmax == 1:
        w[1] = edge * (2 - edge / dq)
    else:
        w[1] = w[-2] = edge * (1 - edge / (2 * dq)) + dq / 2
    return Nr - 1 - rmax, w / (2 * na)


def spectrum(focused, pre, post, q_start, weights):
    """(Ny, Nx, Nl) incoherent spectrum: sum over the weighted wavevectors of
    0.5 * ||post . T . pre||_F^2, T[j][i] = focused[l, q, 2i+j] (:348-388, 511-513)."""
    Nl, Nq, _, Ny, Nx = focused.shape
    out = np.zeros((Ny, Nx, Nl))
    for k, wk in enumerate(weights):
        q = q_start + k
        T = focused[:, q].reshape(Nl, 2, 2, Ny, Nx).transpose(0, 3, 4, 2, 1)  # [l, y, x, j, i]
        M = post[:, None, None] @ (T @ pre[:, None, None])
        sp = 0.5 * np.sum(np.abs(M) ** 2, axis=(-1, -2))
        out += wk * sp.transpose(1, 2, 0)
    return out
