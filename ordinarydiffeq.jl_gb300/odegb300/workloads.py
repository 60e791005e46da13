"""Seeded synthetic ensembles with the shapes of the benchmark configurations,
and the algorithmic FLOP counts the roofline uses.

No public dataset exists for this path; each workload is generated from a seed
with the sizes and parameter distributions of the configuration it names.
"""
import numpy as np

# ---------------------------------------------------------------- workloads


def lorenz(N, seed=42):
    """10k-style Lorenz ensemble: u0 = (1, 0, 0), sigma = 10, beta = 8/3, rho ~ U(0, 21),
    tspan (0, 1), Tsit5, reltol = abstol = 1e-8, saveat 0.1."""
    rng = np.random.default_rng(seed)
    u0 = np.tile(np.array([[1.0], [0.0], [0.0]]), (1, N))
    p = np.vstack([np.full(N, 10.0), rng.uniform(0.0, 21.0, N), np.full(N, 8.0 / 3.0)])
    ts = np.vstack([np.zeros(N), np.ones(N)])
    return dict(model="lorenz", alg="tsit5", u0=u0, p=p, tspan=ts, saveat=0.1, reltol=1e-8, abstol=1e-8)


ROBER_SAVEAT = 10.0 ** np.linspace(-5.0, 5.0, 20)


def robertson(N, seed=42, alg="rodas5p", reltol=1e-6, abstol=1e-10):
    """Robertson kinetics: k = (0.04, 3e7, 1e4) each scaled by 2^U(-1, 1) (log-uniform in
    [0.5, 2]); u0 = (1, 0, 0); tspan (0, 1e5); 20 log-spaced saves in (0, 1e5];
    Rodas5P with the analytic Jacobian, reltol 1e-6, abstol 1e-10 (or the given
    Rosenbrock method and tolerances)."""
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4])[:, None] * 2.0 ** rng.uniform(-1.0, 1.0, (3, N))
    u0 = np.tile(np.array([[1.0], [0.0], [0.0]]), (1, N))
    ts = np.vstack([np.zeros(N), np.full(N, 1e5)])
    return dict(model="robertson", alg=alg, u0=u0, p=p, tspan=ts, saveat=ROBER_SAVEAT, reltol=reltol,
                abstol=abstol)


def bouncing_ball(N, seed=42):
    """Balls dropped from 20-50 m (v0 ~ U(-5, 5)) under g = 9.81 with the model's
    ContinuousCallback (condition x, affect_neg! v <- -e v): restitution e ~
    U(0.85, 0.95), so the bounces stay apart over tspan (0, 10); half of the
    balls terminate! at their first contact after t_stop ~ U(3, 10), the rest
    bounce to tf.  Tsit5, reltol = abstol = 1e-6, saveat 0.25 (41 saves)."""
    from .ensemble import ContinuousCallback
    rng = np.random.default_rng(seed)
    u0 = np.vstack([rng.uniform(20.0, 50.0, N), rng.uniform(-5.0, 5.0, N)])
    t_stop = np.where(rng.uniform(0.0, 1.0, N) < 0.5, rng.uniform(3.0, 10.0, N), 1e9)
    p = np.vstack([np.full(N, 9.81), rng.uniform(0.85, 0.95, N), t_stop])
    ts = np.vstack([np.zeros(N), np.full(N, 10.0)])
    return dict(model="bouncing_ball", alg="tsit5", u0=u0, p=p, tspan=ts, saveat=0.25, reltol=1e-6, abstol=1e-6,
                callback=ContinuousCallback(interp_points=10, max_events=8))


def pk_dosing(N, seed=42):
    """Population pharmacokinetics: a one-compartment model with first-order
    absorption per patient, ka and ke log-normal (medians 1.2 and 0.15 per hour,
    30% spread), a 100 mg dose at t = 0 and then every 12 h for a week by the
    model's DiscreteCallback (condition t in tstops, tstops = the dose times),
    Tsit5, reltol 1e-6, abstol 1e-8, hourly saves."""
    from .ensemble import DiscreteCallback
    rng = np.random.default_rng(seed)
    ka = 1.2 * np.exp(0.3 * rng.standard_normal(N))
    ke = 0.15 * np.exp(0.3 * rng.standard_normal(N))
    dose = np.full(N, 100.0)
    u0 = np.vstack([dose, np.zeros(N)])
    ts = np.vstack([np.zeros(N), np.full(N, 168.0)])
    return dict(model="pk_one_compartment", alg="tsit5", u0=u0, p=np.vstack([ka, ke, dose]), tspan=ts, saveat=1.0,
                reltol=1e-6, abstol=1e-8, tstops=12.0 * np.arange(1, 14), callback=DiscreteCallback(max_events=14))


def van_der_pol(N, seed=42):
    """Van der Pol oscillators (the reference's stiffness-detection problem) with
    mu log-uniform in [1, 1000] (from non-stiff to stiff relaxation), u0 = (2, 0),
    tspan (0, 6), AutoTsit5(Rosenbrock23()), reltol = abstol = 1e-6, saveat 0.5."""
    rng = np.random.default_rng(seed)
    u0 = np.tile(np.array([[2.0], [0.0]]), (1, N))
    p = (10.0 ** rng.uniform(0.0, 3.0, N))[None, :]
    ts = np.vstack([np.zeros(N), np.full(N, 6.0)])
    return dict(model="van_der_pol", alg="autotsit5_rosenbrock23", u0=u0, p=p, tspan=ts, saveat=0.5, reltol=1e-6,
                abstol=1e-6)


def duffing(N, seed=42, sizes=(2, 4, 8, 16, 32), tf_range=(1.0, 100.0)):
    """Uneven Duffing chains: N oscillators uniform in `sizes` (2N states), stiffness and
    damping ~ U(0.1, 1), cubic ~ U(0, 5), u0 ~ N(0, 1), tf log-uniform in tf_range,
    16 uniform saves in (0, tf]; Vern7, reltol = abstol = 1e-6."""
    rng = np.random.default_rng(seed)
    npt = (2 * rng.choice(np.asarray(sizes), N)).astype(np.int32)
    nmax = int(npt.max())
    u0 = rng.standard_normal((nmax, N))
    u0[np.arange(nmax)[:, None] >= npt[None, :]] = 0.0
    p = np.vstack([rng.uniform(0.1, 1.0, N), rng.uniform(0.1, 1.0, N), rng.uniform(0.0, 5.0, N)])
    tf = 10.0 ** rng.uniform(np.log10(tf_range[0]), np.log10(tf_range[1]), N)
    ts = np.vstack([np.zeros(N), tf])
    saveat = np.outer(np.arange(1, 17) / 16.0, tf)
    return dict(model="duffing_chain", alg="vern7", u0=u0, p=p, tspan=ts, saveat=saveat, reltol=1e-6,
                abstol=1e-6, n_per_traj=npt)


def brusselator(N, seed=42, cells=32):
    """Brusselator 1-D, 32 periodic cells (64 states): A ~ U(0.5, 1.5), B ~ U(2, 4),
    alpha log-uniform in [1e-3, 1e-1], u0 = steady state (A, B/A) + 0.1 N(0, 1);
    tspan (0, 10), saves at 1.25:1.25:10; Rodas5P, reltol 1e-5, abstol 1e-8."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(0.5, 1.5, N)
    B = rng.uniform(2.0, 4.0, N)
    alpha = 10.0 ** rng.uniform(-3.0, -1.0, N)
    n = 2 * cells
    u0 = np.empty((n, N))
    u0[0::2] = A[None, :]
    u0[1::2] = (B / A)[None, :]
    u0 += 0.1 * rng.standard_normal((n, N))
    p = np.vstack([A, B, alpha])
    ts = np.vstack([np.zeros(N), np.full(N, 10.0)])
    return dict(model="brusselator_1d", alg="rodas5p", u0=u0, p=p, tspan=ts, saveat=1.25, reltol=1e-5,
                abstol=1e-8, ir_sweeps=1)


# ---------------------------------------------------------------- FLOP model
# Algorithmic floating-point operations per attempted step (an fma counts 2),
# counted from the kernels' own arithmetic.  F: FLOPs of one RHS evaluation.

RHS_FLOPS = {"linear": lambda n: n, "lorenz": lambda n: 9, "robertson": lambda n: 13,
             "duffing_chain": lambda n: 9 * (n // 2), "brusselator_1d": lambda n: 13 * (n // 2),
             "bouncing_ball": lambda n: 1, "van_der_pol": lambda n: 7, "pk_one_compartment": lambda n: 5}
JAC_FLOPS = {"linear": lambda n: 0, "lorenz": lambda n: 3, "robertson": lambda n: 10,
             "duffing_chain": lambda n: 5 * (n // 2), "brusselator_1d": lambda n: 14 * (n // 2),
             "bouncing_ball": lambda n: 0, "van_der_pol": lambda n: 8, "pk_one_compartment": lambda n: 0}
CONTROLLER_FLOPS = 150  # two series pow evaluations, clamp, dt update (FP64)


def error_norm_flops(n):
    return 6 * n + 4


def attempt_flops(alg, model, n):
    F = RHS_FLOPS[model](n)
    if alg == "tsit5":
        # 6 RHS; stage sums 21 fma + solution 6 fma (in the 21) + btilde 7 fma per state
        return 6 * F + n * (2 * 21 + 2 * 7 + 6) + error_norm_flops(n) + CONTROLLER_FLOPS
    if alg == "vern7":
        # 10 RHS; 36 stage fma + 7 solution fma + 8 btilde fma per state
        return 10 * F + n * (2 * 36 + 2 * 7 + 2 * 8 + 10) + error_norm_flops(n) + CONTROLLER_FLOPS
    if alg == "rodas5p":
        Jf = JAC_FLOPS[model](n)
        if model == "brusselator_1d":
            # the kernel's LU skips the zero columns of each pivot row: count the
            # structural nonzeros of the periodic band (and its fill)
            lu = lu_struct_flops(brusselator_pattern(n))
        else:
            lu = sum((n - c - 1) + 2 * (n - c - 1) ** 2 + 1 for c in range(n))
        solve = 2 * n * n + n
        return (8 * F + Jf + 2 * n + lu + 8 * solve + n * (2 * 28 + 2 * 28 + 2 * 8 + 2 * 24) + 28 + 8
                + error_norm_flops(n) + CONTROLLER_FLOPS)
    if alg == "autotsit5_rosenbrock23":   # the Tsit5 attempt (the common one) plus the stiffness estimate
        return attempt_flops("tsit5", model, n) + 3 * n
    if alg == "rosenbrock23":
        # 2 RHS (f at the half step, FSAL f(u)) + J, W, LU, 3 solves; per state the
        # stage, FSAL-difference and error-estimate arithmetic: 19 flops
        Jf = JAC_FLOPS[model](n)
        if model == "brusselator_1d":
            lu = lu_struct_flops(brusselator_pattern(n))
        else:
            lu = sum((n - c - 1) + 2 * (n - c - 1) ** 2 + 1 for c in range(n))
        solve = 2 * n * n + n
        return 2 * F + Jf + 2 * n + lu + 3 * solve + 19 * n + error_norm_flops(n) + CONTROLLER_FLOPS
    raise ValueError(alg)


def brusselator_pattern(n):
    """Structural nonzeros of W = J - I/(dt*gamma) for the periodic Brusselator."""
    nc = n // 2
    P = np.zeros((n, n), dtype=bool)
    for c in range(nc):
        for d in (c - 1, c, c + 1):
            d %= nc
            P[2 * c, 2 * d] = P[2 * c + 1, 2 * d + 1] = True
        P[2 * c, 2 * c + 1] = P[2 * c + 1, 2 * c] = True
    return P


def lu_struct_flops(P):
    """FLOPs of an LU without row exchanges that skips zero multipliers and zero
    pivot-row entries (one division per multiplier, one fma per update)."""
    P = P.copy()
    n = P.shape[0]
    fl = 0
    for c in range(n):
        rows = np.nonzero(P[c + 1:, c])[0] + c + 1
        cols = np.nonzero(P[c, c + 1:])[0] + c + 1
        fl += 1 + len(rows) + 2 * len(rows) * len(cols)
        P[np.ix_(rows, cols)] = True
    return fl


def save_flops(alg, model, n):
    """Extra work of a step that holds saveat points (Vern7 lazy stages + interpolant)."""
    F = RHS_FLOPS[model](n)
    if alg == "vern7":
        return 6 * F + n * 2 * (7 + 8 + 9 + 10 + 10 + 10) + n * 2 * 13
    if alg == "tsit5":
        return n * 2 * 7
    if alg == "rosenbrock23":
        return n * 2 * 2 + 8
    if alg == "autotsit5_rosenbrock23":
        return n * 2 * 7
    return n * 2 * 5
