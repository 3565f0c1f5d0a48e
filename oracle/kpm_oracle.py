"""CPU oracle for the KPM hot path: a numpy/scipy restatement of kwant.kpm.

TEST INFRASTRUCTURE ONLY.  Nothing in the ``kwant_gb300`` package imports
this module; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg use it, and only as the checker / the timed CPU reference.

Each function restates one piece of the reference algorithm and cites the
reference file:line it follows (paths relative to the Kwant source tree).
The oracle is pinned against golden vectors produced by running the
reference itself (``tests/golden/make_golden.py``), see
``tests/test_oracle_golden.py``.

Third-party numerics on the path (not part of the reference tree, unpinned in
its ``setup.cfg:33-36``): scipy's ``fftpack.dct`` (type III, pocketfft),
ARPACK ``eigsh`` and ``integrate.simpson``; the oracle calls the same scipy
routines (scipy 1.18 here) so that it agrees with the reference to rounding.
"""

import math

import numpy as np
import scipy.fftpack as _fft
import scipy.sparse as sp
from scipy.integrate import simpson
from scipy.sparse.linalg import eigsh

SAMPLING = 2  # kwant/kpm.py:36


# --------------------------------------------------------------------------
# Random vectors and rescaling
# --------------------------------------------------------------------------

def ensure_rng(rng=None):
    """kwant/_common.py:115-135: None -> numpy global, int -> RandomState."""
    if rng is None:
        return np.random.mtrand._rand
    if isinstance(rng, (int, np.integer)):
        return np.random.RandomState(rng)
    return rng


def draw_v0(rng, n):
    """kwant/kpm.py:201-203: the vector stored for reproducibility and used
    as ARPACK's starting vector; the first ``n`` draws of the stream."""
    return np.exp(2j * np.pi * rng.random_sample(n))


def random_vectors(rng, n, count, orbs=None):
    """kwant/kpm.py:932-951 (``RandomVectors``): each vector consumes the
    next ``len(orbs)`` draws of the stream; zeros outside ``orbs``."""
    out = np.zeros((count, n), dtype=complex)
    idx = np.arange(n) if orbs is None else np.asarray(orbs)
    for r in range(count):
        out[r, idx] = np.exp(2j * np.pi * rng.random_sample(len(idx)))
    return out


def spectral_bounds(ham, eps, v0):
    """kwant/kpm.py:1166-1172: extremal eigenvalues by ARPACK, tol = eps/2."""
    tol = eps / 2
    lmax = eigsh(ham, k=1, which='LA', return_eigenvectors=False,
                 tol=tol, v0=v0)[0]
    lmin = eigsh(ham, k=1, which='SA', return_eigenvectors=False,
                 tol=tol, v0=v0)[0]
    return lmin, lmax


def rescale_ab(lmin, lmax, eps):
    """kwant/kpm.py:1174-1180: a = |lmax-lmin|/(2-eps), b = midpoint, with
    the single-eigenvalue guard."""
    tol = eps / 2
    a = np.abs(lmax - lmin) / (2. - eps)
    b = (lmax + lmin) / 2.
    if lmax - lmin <= abs(lmax + lmin) * tol / 2:
        raise ValueError('The Hamiltonian has a single eigenvalue, it is not '
                         'possible to obtain a spectral density.')
    return a, b


def rescaled_matvec(ham, a, b, v):
    """kwant/kpm.py:1182-1183: (H v - b v) / a, H not rescaled in place."""
    return (ham.dot(v) - b * v) / a


# --------------------------------------------------------------------------
# Chebyshev recursion (the hot loop)
# --------------------------------------------------------------------------

def moments_dos(ham, a, b, alpha0, num_moments, state=None, prev=None):
    """Moments of one vector with operator=None, kwant/kpm.py:436-477.

    Uses the doubling identities mu_2n = 2<a_n|a_n> - mu_0 and
    mu_2n+1 = 2<a_n+1|a_n> - mu_1 (one matvec per two moments).  ``state``
    resumes from (alpha_{n-1}, alpha_n) and the old moments ``prev``
    (kwant/kpm.py:449-452).  Returns (moments, (alpha, alpha_next)).
    """
    ham = sp.csr_matrix(ham)
    mom = [0.] * num_moments
    if state is None:
        alpha = alpha0
        alpha_next = rescaled_matvec(ham, a, b, alpha)
        mom[0] = np.vdot(alpha0, alpha0)
        mom[1] = np.vdot(alpha0, alpha_next)
        m_start = 2
    else:
        alpha, alpha_next = state
        m_start = len(prev)
        mom[:m_start] = list(prev)
    for n in range(m_start // 2, num_moments // 2):
        alpha_save = alpha_next
        alpha_next = 2 * rescaled_matvec(ham, a, b, alpha_next) - alpha
        alpha = alpha_save
        mom[2 * n] = 2 * np.vdot(alpha, alpha) - mom[0]
        mom[2 * n + 1] = 2 * np.vdot(alpha_next, alpha) - mom[1]
    if num_moments % 2:
        mom[num_moments - 1] = 2 * np.vdot(alpha_next, alpha_next) - mom[0]
    return mom, (alpha, alpha_next)


def moments_operator(ham, a, b, alpha0, num_moments, op, state=None,
                     prev=None):
    """Moments of one vector with a sesquilinear ``op(bra, ket)``,
    kwant/kpm.py:439-448 and :478-484: mu_n = op(alpha_0, T_n(H) alpha_0)."""
    ham = sp.csr_matrix(ham)
    mom = [0.] * num_moments
    if state is None:
        alpha = alpha0
        alpha_next = rescaled_matvec(ham, a, b, alpha)
        mom[0] = op(alpha0, alpha0)
        mom[1] = op(alpha0, alpha_next)
        m_start = 2
    else:
        alpha, alpha_next = state
        m_start = len(prev)
        mom[:m_start] = list(prev)
    for n in range(m_start, num_moments):
        alpha_save = alpha_next
        alpha_next = 2 * rescaled_matvec(ham, a, b, alpha_next) - alpha
        alpha = alpha_save
        mom[n] = op(alpha0, alpha_next)
    return mom, (alpha, alpha_next)


def chebyshev_vectors(ham, a, b, alpha0, num_moments):
    """T_n(H~)|alpha_0> for n < num_moments: the 'moments' a fake operator
    ``op(bra, ket) = ket`` records in kwant/kpm.py:570-575."""
    ham = sp.csr_matrix(ham)
    out = np.empty((num_moments, alpha0.shape[0]), dtype=complex)
    alpha = alpha0
    out[0] = alpha0
    if num_moments == 1:
        return out
    alpha_next = rescaled_matvec(ham, a, b, alpha)
    out[1] = alpha_next
    for n in range(2, num_moments):
        alpha_save = alpha_next
        alpha_next = 2 * rescaled_matvec(ham, a, b, alpha_next) - alpha
        alpha = alpha_save
        out[n] = alpha_next
    return out


# --------------------------------------------------------------------------
# Kernels and reconstruction
# --------------------------------------------------------------------------

def jackson_kernel(moments):
    """kwant/kpm.py:1106-1123 (Rev. Mod. Phys. 78, 275, Eq. 71)."""
    n = len(moments)
    m = np.arange(n)
    g = ((n - m + 1) * np.cos(np.pi * m / (n + 1)) +
         np.sin(np.pi * m / (n + 1)) / np.tan(np.pi / (n + 1)))
    g /= n + 1
    return np.transpose(np.transpose(moments) * g)


def lorentz_kernel(moments, l=4):
    """kwant/kpm.py:1126-1142."""
    n = len(moments)
    m = np.arange(n)
    g = np.sinh(l * (1 - m / n)) / np.sinh(l)
    return np.transpose(np.transpose(moments) * g)


def chebyshev_nodes(n_sampling):
    """kwant/kpm.py:1190-1194: ascending nodes cos(pi (k+1/2) / n)."""
    raw, step = np.linspace(np.pi, 0, n_sampling, endpoint=False,
                            retstep=True)
    return np.cos(raw + step / 2)


def calc_fft_moments(moments):
    """kwant/kpm.py:1197-1222: zero-pad to 2M, DCT-III, reverse to ascending
    energies, divide by pi*sqrt(1-x^2).  Returns (rho, gammas)."""
    moments = np.asarray(moments)
    n_moments, *extra = moments.shape
    n_sampling = SAMPLING * n_moments
    ext = np.zeros([n_sampling] + extra, dtype=moments.dtype)
    x = chebyshev_nodes(n_sampling)
    ext[:n_moments] = moments
    gammas = np.transpose(_fft.dct(ext.transpose(), type=3))[::-1]
    gk = np.pi * np.sqrt(1 - x ** 2)
    rho = np.transpose(np.divide(gammas.transpose(), gk))
    return rho, gammas


def reduce_moments(moments_list, a, mean=True, kernel=jackson_kernel):
    """kwant/kpm.py:378-388: real_if_close, vector axis second, mean, /a,
    kernel."""
    moments = np.real_if_close(moments_list)
    moments = np.swapaxes(moments, 0, 1)
    if mean:
        moments = np.mean(moments, axis=1)
    moments = moments / a
    return kernel(moments)


def energies(a, b, num_moments):
    """kwant/kpm.py:254-257."""
    return a * chebyshev_nodes(SAMPLING * num_moments) + b


def spectral_density(ham, vectors, lmin, lmax, num_moments, eps=0.05,
                     op=None, mean=True, kernel=jackson_kernel):
    """The whole SpectralDensity pipeline on explicit vectors and bounds
    (kwant/kpm.py:163-252).  Returns a dict of the reference's state."""
    a, b = rescale_ab(lmin, lmax, eps)
    mlist = []
    for v in vectors:
        if op is None:
            mom, _ = moments_dos(ham, a, b, v, num_moments)
        else:
            mom, _ = moments_operator(ham, a, b, v, num_moments, op)
        mlist.append(mom)
    mom = reduce_moments(mlist, a, mean=mean, kernel=kernel)
    rho, gam = calc_fft_moments(mom)
    return dict(a=a, b=b, moments_list=np.array(mlist), densities=rho,
                gammas=gam, energies=energies(a, b, num_moments))


def evaluate(moments, a, b, energy):
    """SpectralDensity.__call__(energy), kwant/kpm.py:285-295 (chebval)."""
    from numpy.polynomial.chebyshev import chebval
    energy = np.asarray(energy)
    e = (energy - b) / a
    g_e = np.pi * np.sqrt(1 - e) * np.sqrt(1 + e)
    moments = np.array(moments, copy=True)
    moments[1:] = 2 * moments[1:]
    return np.transpose(chebval(e, moments) / g_e)


def integrate(gammas, a, num_moments, energies_=None, distribution=None):
    """SpectralDensity.integrate, kwant/kpm.py:297-316 (Gauss-Chebyshev)."""
    factor = a / (2 * num_moments)
    if distribution is None:
        rho = gammas
    else:
        rho = np.transpose(gammas.transpose() * distribution(energies_))
    return factor * np.sum(rho, axis=0)


# --------------------------------------------------------------------------
# Local operators (MAT_ELS / ACT), restated with numpy
# --------------------------------------------------------------------------

def site_orbitals(site_ranges, sites):
    """kwant/operator.pyx:114-125 (``_get_orbs``): first orbital and norbs
    of each site, by bisection over ``site_ranges`` rows (first_site,
    norbs, orb_offset)."""
    sr = np.asarray(site_ranges, dtype=np.int64)
    sites = np.asarray(sites, dtype=np.int64)
    run = np.searchsorted(sr[:, 0], sites, side='right') - 1
    norbs = sr[run, 1]
    start = sr[run, 2] + (sites - sr[run, 0]) * norbs
    return start, norbs


def density_matels(bra, ket, site_ranges, where, onsite_blocks, sum_=False,
                   real=False):
    """Density MAT_ELS, kwant/operator.pyx:785-807:
    q_w = sum_ij conj(bra[a_s+i]) M_w[i,j] ket[a_s+j].

    ``onsite_blocks`` is a list (one norbs x norbs matrix per where-site) or
    a single matrix used everywhere.  ``real`` reproduces the `.real` of
    kwant/operator.pyx:556-558."""
    start, norbs = site_orbitals(site_ranges, where)
    out = np.zeros(len(where), dtype=complex)
    for w in range(len(where)):
        M = onsite_blocks if not isinstance(onsite_blocks, list) \
            else onsite_blocks[w]
        M = np.asarray(M, dtype=complex)
        n = norbs[w]
        M = M[:n, :n] if M.shape[0] > n else M
        s = start[w]
        out[w] = np.conj(bra[s:s + n]) @ M @ ket[s:s + n]
    if real:
        out = out.real
    return np.sum(out) if sum_ else out


def current_matels(bra, ket, site_ranges, hoppings, hop_blocks,
                   onsite_blocks, sum_=False, real=False):
    """Current MAT_ELS, kwant/operator.pyx:977-987:
    J_w = i sum [conj(bra_b) H_ab^dagger M_a ket_a - conj(bra_a) M_a H_ab ket_b]
    for hopping w = (a, b) with H_ab the (a_norbs x b_norbs) block."""
    hoppings = np.asarray(hoppings)
    a_s, a_n = site_orbitals(site_ranges, hoppings[:, 0])
    b_s, b_n = site_orbitals(site_ranges, hoppings[:, 1])
    out = np.zeros(len(hoppings), dtype=complex)
    for w in range(len(hoppings)):
        H = np.asarray(hop_blocks[w], dtype=complex)
        M = onsite_blocks if not isinstance(onsite_blocks, list) \
            else onsite_blocks[w]
        M = np.asarray(M, dtype=complex)
        na, nb = a_n[w], b_n[w]
        M = M[:na, :na] if M.shape[0] > na else M
        ka = ket[a_s[w]:a_s[w] + na]
        kb = ket[b_s[w]:b_s[w] + nb]
        ba = bra[a_s[w]:a_s[w] + na]
        bb = bra[b_s[w]:b_s[w] + nb]
        tmp = (np.conj(bb) @ H.conj().T @ M @ ka
               - np.conj(ba) @ M @ H @ kb)
        out[w] = 1j * tmp
    if real:
        out = out.real
    return np.sum(out) if sum_ else out


def source_matels(bra, ket, site_ranges, where, ham_blocks, onsite_blocks,
                  sum_=False, real=False):
    """Source MAT_ELS, kwant/operator.pyx:1091-1104:
    q_w = i sum_i conj(bra[a_s+i]) [(H_aa^dagger M_a - M_a H_aa) ket_a]_i
    for site w = a, with H_aa the onsite block of the Hamiltonian."""
    start, norbs = site_orbitals(site_ranges, where)
    out = np.zeros(len(where), dtype=complex)
    for w in range(len(where)):
        M = onsite_blocks if not isinstance(onsite_blocks, list) \
            else onsite_blocks[w]
        M = np.asarray(M, dtype=complex)
        n = norbs[w]
        M = M[:n, :n] if M.shape[0] > n else M
        H = np.asarray(ham_blocks[w], dtype=complex)
        s = start[w]
        k = ket[s:s + n]
        out[w] = 1j * (np.conj(bra[s:s + n]) @ (H.conj().T @ M @ k
                                                 - M @ H @ k))
    if real:
        out = out.real
    return np.sum(out) if sum_ else out


def source_act(ket, site_ranges, where, ham_blocks, onsite_blocks):
    """Source ACT, kwant/operator.pyx:1105-1115:
    out[a_s+i] += i [(H_aa^dagger M_a - M_a H_aa) ket_a]_i."""
    start, norbs = site_orbitals(site_ranges, where)
    out = np.zeros(len(ket), dtype=complex)
    for w in range(len(where)):
        M = onsite_blocks if not isinstance(onsite_blocks, list) \
            else onsite_blocks[w]
        M = np.asarray(M, dtype=complex)
        n = norbs[w]
        H = np.asarray(ham_blocks[w], dtype=complex)
        s = start[w]
        k = ket[s:s + n]
        out[s:s + n] += 1j * (H.conj().T @ M @ k - M @ H @ k)
    return out


# --------------------------------------------------------------------------
# Correlator / Kubo-Bastin conductivity
# --------------------------------------------------------------------------

def velocity(ham, positions, direction):
    """kwant/kpm.py:1042-1085 (``_velocity`` for a matrix Hamiltonian and
    per-orbital positions): v = H o i (x_col - x_row); explicit zeros of the
    COO product are kept."""
    op = sp.coo_matrix(ham, copy=True)
    disp = positions[op.col] - positions[op.row]
    op.data = op.data * (1j * disp[:, direction])
    return op.tocsr()


def correlator_moments_matrix(ham, vectors, lmin, lmax, num_moments,
                              op_alpha, op_beta, eps=0.05, mean=True):
    """Correlator.__init__ + _calculate_moments_matrix,
    kwant/kpm.py:557-606 and :685-695.

    Psi[r, :, n] = op_beta T_n(H~)|r>,  Omega[r, m, :] = T_m(H~) op_alpha|r>,
    mu = Omega^* @ Psi (mean over r).  The second SpectralDensity is given
    bounds (b -+ a(1 - eps/2)), which reproduce the same (a, b)
    (kwant/kpm.py:576-579); that arithmetic is reproduced here."""
    op_alpha = sp.csr_matrix(op_alpha)
    op_beta = sp.csr_matrix(op_beta)
    a, b = rescale_ab(lmin, lmax, eps)
    _a = a * (1 - eps / 2)
    a2, b2 = rescale_ab(b - _a, b + _a, eps)
    mus = []
    for v in vectors:
        tr = chebyshev_vectors(ham, a, b, v, num_moments)
        psi = np.array([op_beta.dot(t) for t in tr]).T          # (N, M)
        tl = chebyshev_vectors(ham, a2, b2, op_alpha.dot(v), num_moments)
        mus.append(tl.conj() @ psi)                               # (M, M)
    mus = np.array(mus)
    mu = np.mean(mus, axis=0) if mean else mus
    return mu, (a, b), (a2, b2)


def integral_factor(mu, a, b, num_moments, kernel=jackson_kernel):
    """Correlator._build_integral_factor, kwant/kpm.py:720-760."""
    g = kernel(np.ones(num_moments))
    g[0] /= 2
    mu_k = np.outer(g, g) * mu
    e_scaled = (energies(a, b, num_moments) - b) / a
    m = np.arange(num_moments)
    out = []
    for e in e_scaled:
        sqrt_e = np.sqrt(1 - e ** 2)
        arccos_e = np.arccos(e)
        exp_n = np.exp(1j * arccos_e * m)
        t_n = np.real(exp_n)
        e_plus = (e - 1j * sqrt_e * m) * exp_n
        big = e_plus[None, :] * t_n[:, None]
        big += big.conj().T
        out.append(np.tensordot(mu_k, big.T))
    return np.array(out).T


def fermi_distribution(energy, mu, temperature):
    """kwant/kpm.py:990-1009."""
    if temperature < 0:
        raise ValueError("temperature must be non-negative")
    elif temperature == 0:
        return np.array(np.less(energy - mu, 0), dtype=float)
    return 1 / (1 + np.exp((energy - mu) / temperature))


def conductivity_value(factor, a, b, num_moments, mu=0, temperature=0):
    """Correlator.__call__, kwant/kpm.py:608-630 (Simpson over the nodes)."""
    e = energies(a, b, num_moments)
    e_r = (e - b) / a
    dist = fermi_distribution(e, mu, temperature)
    integrand = np.divide(dist, (1 - e_r ** 2) ** 2)
    integrand = np.multiply(integrand, factor)
    integral = simpson(integrand, x=e_r)
    return 2 * 4 ** 2 / ((2 * a) ** 2) * integral


def energy_resolution_moments(a, energy_resolution):
    """kwant/kpm.py:216-217 and :346."""
    return math.ceil((1.6 * a) / energy_resolution)
