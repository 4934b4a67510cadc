"""Material parameters and state construction for the GPR model.

`Par` mirrors the reference's `GPRpy.classes.Par` (code/cpp/src/system/objects.h:22-98)
for the fields the GPR time step reads, and `material_params` restates the
reference's builder (code/python/gpr/misc/objects.py:184-267) with the same
defaults: n=1 (Newtonian) unless given, beta=0, pINF=0 when gamma is given,
kappa = mu*gamma*cv/Pr when Pr is given, calpha2 = calpha**2, b02 = b0**2,
Tref = 0, no body force and no reaction.

`Par.to_ctypes()` packs the fields into the `gpr_par` C struct declared in
include/gpr_gb300.h; the same layout is used by the CUDA library and the oracle.
"""
import ctypes

import numpy as np

# EOS codes of the reference (code/cpp/src/system/energy/mg.h:6-11).
VACUUM = -1
STIFFENED_GAS = 0
SHOCK_MG = 1
JWL = 2
COCHRAN_CHAN = 3
GODUNOV_ROMENSKI = 4

EOS_CODES = {"sg": STIFFENED_GAS, "smg": SHOCK_MG, "jwl": JWL,
             "cc": COCHRAN_CHAN, "gr": GODUNOV_ROMENSKI, "vac": VACUUM}

FLAG_SOLID = 1
FLAG_POWER_LAW = 2
FLAG_BINGHAM = 4

_DOUBLE_FIELDS = ("rho0", "Tref", "cv", "pINF", "Gamma0", "c02", "s", "alpha",
                  "beta", "gamma", "A", "B", "R1", "R2", "b02", "mu", "tau0",
                  "sigmaY", "n", "calpha2", "kappa")


class GprParC(ctypes.Structure):
    """ctypes image of `gpr_par` (include/gpr_gb300.h)."""
    _fields_ = ([("EOS", ctypes.c_int32), ("flags", ctypes.c_int32)]
                + [(f, ctypes.c_double) for f in _DOUBLE_FIELDS]
                + [("dp", ctypes.c_double * 3)])


class Par:
    """Material parameters of one GPR material (reference `classes.Par`)."""

    def __init__(self):
        self.EOS = 0
        self.SOLID = False
        self.POWER_LAW = False
        self.BINGHAM = False
        for f in _DOUBLE_FIELDS:
            setattr(self, f, 0.0)
        self.dp = np.zeros(3)
        self.REACTION = -1

    @property
    def flags(self):
        return ((FLAG_SOLID if self.SOLID else 0)
                | (FLAG_POWER_LAW if self.POWER_LAW else 0)
                | (FLAG_BINGHAM if self.BINGHAM else 0))

    def to_ctypes(self):
        c = GprParC()
        c.EOS = int(self.EOS)
        c.flags = self.flags
        for f in _DOUBLE_FIELDS:
            setattr(c, f, float(getattr(self, f)))
        for i in range(3):
            c.dp[i] = float(self.dp[i])
        return c

    def to_array(self):
        """Flat float64 image used by the batched form's per-instance table."""
        c = self.to_ctypes()
        return np.frombuffer(bytes(c), dtype=np.uint8).copy()

    @classmethod
    def from_array(cls, arr):
        """Inverse of `to_array`."""
        c = GprParC.from_buffer_copy(np.asarray(arr, dtype=np.uint8).tobytes())
        p = cls()
        p.EOS = c.EOS
        p.SOLID = bool(c.flags & FLAG_SOLID)
        p.POWER_LAW = bool(c.flags & FLAG_POWER_LAW)
        p.BINGHAM = bool(c.flags & FLAG_BINGHAM)
        for f in _DOUBLE_FIELDS:
            setattr(p, f, getattr(c, f))
        p.dp = np.array([c.dp[0], c.dp[1], c.dp[2]])
        return p

    def copy(self):
        p = Par()
        p.__dict__.update({k: (v.copy() if isinstance(v, np.ndarray) else v)
                           for k, v in self.__dict__.items()})
        return p

    def __repr__(self):
        keys = ["EOS", "rho0", "cv", "gamma", "pINF", "b02", "mu", "n",
                "calpha2", "kappa"]
        return "Par(%s)" % ", ".join("%s=%r" % (k, getattr(self, k)) for k in keys)


def material_params(EOS, rho0, cv=None, Tref=None, alpha=None, beta=None,
                    gamma=None, pINF=None, c0=None, Gamma0=None, s=None,
                    A=None, B=None, R1=None, R2=None, b0=None, mu=None,
                    tau0=None, sigmaY=None, n=None, calpha=None, kappa=None,
                    Pr=None, dp=None):
    """Build a `Par` exactly as code/python/gpr/misc/objects.py:184-267 does
    (single material, no reaction, no mixture)."""
    MP = Par()
    if EOS == "vac":
        MP.EOS = VACUUM
        return MP
    if Tref is None:
        Tref = 0
    if gamma and pINF is None:
        pINF = 0
    if n:
        POWER_LAW = True
        SOLID = bool(sigmaY)
        BINGHAM = False
    else:
        n = 1
        POWER_LAW = False
        SOLID = not mu
        BINGHAM = bool(mu and sigmaY)
    if beta is None:
        beta = 0
    if Pr:
        kappa = mu * gamma * cv / Pr

    MP.EOS = EOS_CODES[EOS]
    MP.rho0 = rho0
    if cv:
        MP.cv = cv
        MP.Tref = Tref
    if EOS == "sg":
        MP.gamma = gamma
        MP.pINF = pINF
    elif EOS == "smg":
        MP.Gamma0 = Gamma0
        MP.c02 = c0 ** 2
        MP.s = s
    elif EOS == "gr":
        MP.c02 = c0 ** 2
        MP.alpha = alpha
        MP.beta = beta
        MP.gamma = gamma
    elif EOS in ("jwl", "cc"):
        MP.Gamma0 = Gamma0
        MP.A = A
        MP.B = B
        MP.R1 = R1
        MP.R2 = R2
    if b0:
        MP.b02 = b0 ** 2
        MP.beta = beta
        MP.POWER_LAW = POWER_LAW
        MP.SOLID = SOLID
        MP.BINGHAM = BINGHAM
        if mu:
            MP.mu = mu
        if n:
            MP.n = n
        if sigmaY:
            MP.sigmaY = sigmaY
        if tau0:
            MP.tau0 = tau0
    if calpha:
        MP.calpha2 = calpha ** 2
        MP.kappa = kappa
    MP.dp = np.zeros(3) if dp is None else np.asarray(dp, dtype=np.float64)
    return MP


# ---------------------------------------------------------------------------
# primitive -> conserved (code/python/gpr/misc/structures.py:104-126 with the
# energy split of code/cpp/src/system/energy/eos.cpp:10-70)

def _gamma_mg(rho, MP):
    if MP.EOS == STIFFENED_GAS:
        return MP.gamma - 1
    if MP.EOS == SHOCK_MG:
        return MP.Gamma0 * MP.rho0 / rho
    if MP.EOS == GODUNOV_ROMENSKI:
        return MP.gamma
    return MP.Gamma0


def _p_ref(rho, MP):
    if MP.EOS == STIFFENED_GAS:
        return -MP.pINF
    if MP.EOS == SHOCK_MG:
        r0 = MP.rho0
        if rho > r0:
            tmp = 1 / r0 - MP.s * (1 / r0 - 1 / rho)
            return MP.c02 * (1 / r0 - 1 / rho) / (tmp * tmp)
        return MP.c02 * (rho - r0)
    if MP.EOS == GODUNOV_ROMENSKI:
        tmp = (rho / MP.rho0) ** MP.alpha
        return MP.c02 * rho / MP.alpha * (tmp - 1) * tmp
    v_ = MP.rho0 / rho
    if MP.EOS == JWL:
        return MP.A * np.exp(-MP.R1 * v_) + MP.B * np.exp(-MP.R2 * v_)
    return MP.A * v_ ** (-MP.R1) - MP.B * v_ ** (-MP.R2)


def _e_ref(rho, MP):
    if MP.EOS == STIFFENED_GAS:
        return MP.pINF / rho
    if MP.EOS == SHOCK_MG:
        return 0.5 * _p_ref(rho, MP) * (1 / MP.rho0 - 1 / rho) if rho > MP.rho0 else 0.0
    if MP.EOS == GODUNOV_ROMENSKI:
        tmp = (rho / MP.rho0) ** MP.alpha
        return MP.c02 / (2 * MP.alpha ** 2) * (tmp - 1) ** 2
    v_ = MP.rho0 / rho
    r0 = MP.rho0
    if MP.EOS == JWL:
        return (MP.A / (r0 * MP.R1) * np.exp(-MP.R1 * v_)
                + MP.B / (r0 * MP.R2) * np.exp(-MP.R2 * v_))
    return (-MP.A / (r0 * (1 - MP.R1)) * (v_ ** (1 - MP.R1) - 1)
            + MP.B / (r0 * (1 - MP.R2)) * (v_ ** (1 - MP.R2) - 1))


def _devGsq(A):
    G = A @ A.T
    t = np.trace(G) / 3
    D = G - t * np.eye(3)
    return float(np.sum(D * D))


def total_energy(rho, p, v, MP, A=None, J=None):
    """E = E_1 + E_2A + E_2J + E_3 (eos.cpp:10-54)."""
    E = _e_ref(rho, MP) + (p - _p_ref(rho, MP)) / (rho * _gamma_mg(rho, MP))
    if A is not None:
        cs2 = MP.b02 * (rho / MP.rho0) ** MP.beta
        C0 = (1 - MP.beta / _gamma_mg(rho, MP)) * cs2
        E += C0 / 4 * _devGsq(np.asarray(A, dtype=np.float64))
    if J is not None:
        E += MP.calpha2 * float(np.dot(J, J)) / 2
    E += float(np.dot(v, v)) / 2
    return E


def Cvec(rho, p, v, MP, A=None, J=None):
    """Conserved vector from primitives, same layout as the reference:
    [rho, rho E, rho v(3), A (9, row-major), rho J (3)]."""
    v = np.asarray(v, dtype=np.float64)
    nv = 5 + (9 if A is not None else 0) + (3 if J is not None else 0)
    Q = np.zeros(nv)
    Q[0] = rho
    Q[1] = rho * total_energy(rho, p, v, MP, A, J)
    Q[2:5] = rho * v
    if A is not None:
        Q[5:14] = np.asarray(A, dtype=np.float64).ravel()
    if J is not None:
        Q[14:17] = rho * np.asarray(J, dtype=np.float64)
    return Q
