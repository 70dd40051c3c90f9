"""Known answers for a plane wave at normal incidence on a slab, for the
slab known-answer tests (test infrastructure, not part of the product).

A plane wave along z in a grid that is periodic along x and y, excited by an
Ex current sheet that spans the whole period, keeps Ex and Hy uniform in x
and y; the 3-D Yee update then is the 1-D one along z: Ex at the integer
nodes k (its medium eps_k, mu = 1), Hy at k + 1/2.  For a time dependence
exp(j w t) sampled at E times n dt and H times (n + 1/2) dt the two updates
read, with a = 2 j sin(w dt / 2) / dt,
    eps_k a E_k       = -(H_{k+1/2} - H_{k-1/2}) / dx
    a H_{k-1/2}       = -(E_k - E_{k-1}) / dx,
and in vacuum E_k = A z0^k + B z0^-k with z0 = exp(-j kappa dx),
sin(kappa dx / 2) = (dx / dt) sin(w dt / 2) (the scheme's own dispersion).
slab_rt_discrete solves these recurrences through the slab exactly: the
power reflection and transmission that the time stepper itself must give,
whatever the resolution.  eps_k of a dispersive node is the susceptibility
that the auxiliary-equation update realises at w (Medium.get_dis_epsilon,
the reference's ffip/geom.py:220-227, 252-260).

slab_rt_airy is the continuum answer (the formulas of the reference's
scripts/basic tests/plane_wave_fic.py:32-42, Airy's two-interface sum),
which the stepper approaches at second order as dx -> 0."""
import numpy as np


def slab_rt_discrete(eps_nodes, f, dt, dx):
    """eps_nodes: permittivity of the slab's E nodes in order of z (vacuum
    on both sides); f: one frequency.  Returns (R, T) as power ratios."""
    eps_nodes = np.asarray(eps_nodes, dtype=complex)
    n = len(eps_nodes)
    w = 2 * np.pi * f
    a = 2j * np.sin(w * dt / 2) / dt
    kappa = 2 * np.arcsin(np.sin(w * dt / 2) * dx / dt) / dx
    z0 = np.exp(-1j * kappa * dx)
    # right of the slab: the transmitted wave alone, E_k = z0^k (k >= n)
    e = z0 ** n
    h = -(z0 ** (n + 1) - e) / (a * dx)  # H_{n+1/2}
    en = {n: e}
    for k in range(n, -2, -1):  # from (E_k, H_{k+1/2}) to (E_{k-1}, H_{k-1/2})
        eps = eps_nodes[k] if 0 <= k < n else 1.0
        h = h + eps * a * dx * e
        e = e + a * dx * h
        en[k - 1] = e
    # left of the slab (k = -1, -2): E_k = A z0^k + B z0^-k
    m = np.array([[z0 ** -1, z0], [z0 ** -2, z0 ** 2]])
    A, B = np.linalg.solve(m, np.array([en[-1], en[-2]]))
    return abs(B / A) ** 2, abs(1 / A) ** 2


def slab_rt_airy(eps, f, d):
    """Continuum power reflection / transmission of a slab of thickness d
    and permittivity eps (mu = 1) in vacuum."""
    eta = np.sqrt(1 / np.asarray(eps, dtype=complex))
    k = 2 * np.pi * np.asarray(f) * np.sqrt(np.asarray(eps, dtype=complex))
    r1 = (eta - 1) / (eta + 1)
    r2 = -r1
    ph = np.exp(-2j * k * d)
    rt = (r1 + r2 * ph) / (1 + r1 * r2 * ph)
    tt = (1 + r1) * (1 + r2) * np.exp(-1j * k * d) / (1 + r1 * r2 * ph)
    return np.abs(rt) ** 2, np.abs(tt) ** 2
