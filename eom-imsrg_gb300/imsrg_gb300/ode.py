"""The traditional IMSRG(2) flow dH/ds = [eta(s), H(s)] (decouple_hamiltonian, src/IMSRG_ODE.f90:9-178).

The reference integrates the vectorized Hamiltonian with the variable-order, variable-step Adams
predictor-corrector code of Shampine and Gordon (L. F. Shampine, M. K. Gordon, Computer Solution
of Ordinary Differential Equations: The Initial Value Problem, Freeman 1975), in its Fortran 90
form in src/adams_ode.f90 (ode :33-247, de :249-595, step :597-1230, intrp :1232-1357).
`AdamsIntegrator` restates that algorithm on NumPy vectors: the same order and step selection,
error estimates, round-off control and interpolation to the output point, with the state that
`ode` keeps in its work arrays carried between calls.  The derivative, one generator and one
commutator, runs on the device through the C ABI; the integrator's vector work (a few dozen
passes over the vector per step) stays on the host.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from .engine import Engine

_EPS = float(np.finfo(np.float64).eps)
_GSTR = np.array([0.0, 0.5, 0.0833, 0.0417, 0.0264, 0.0188, 0.0143, 0.0114, 0.00936, 0.00789, 0.00679,
                  0.00592, 0.00524, 0.00468])           # 1-based: gstr(1..13)
_TWO = np.array([0.0] + [2.0 ** i for i in range(1, 14)])  # two(1..13) = 2, 4, ..., 8192


class AdamsIntegrator:
    """Shampine-Gordon Adams PECE integration of y' = f(t, y) with relative / absolute error
    control; `integrate(t, tout, y)` advances like one call of the reference's `ode` with
    iflag = 1 on the first call and the returned iflag afterwards.  Indices below are 1-based
    as in the published algorithm (element 0 of each small array is unused)."""

    MAXNUM = 500

    def __init__(self, f, neq: int, relerr: float, abserr: float):
        self.f, self.neq = f, int(neq)
        self.relerr, self.abserr = float(relerr), float(abserr)
        n = self.neq
        self.yy, self.wt, self.p = np.zeros(n), np.zeros(n), np.zeros(n)
        self.yp, self.ypout = np.zeros(n), np.zeros(n)
        self.phi = np.zeros((17, n))
        self.alpha, self.beta, self.v, self.w, self.psi = (np.zeros(13) for _ in range(5))
        self.sig, self.g = np.zeros(14), np.zeros(14)
        self.x = self.h = self.hold = self.told = self.delsgn = 0.0
        self.ns = self.k = self.kold = self.isnold = 0
        self.start = self.phase1 = self.nornd = False
        self.iflag = 1
        self.evaluations = 0
        self.steps = 0

    def _f(self, x, y):
        self.evaluations += 1
        return self.f(x, y)

    # ------------------------------------------------------------------ de (src/adams_ode.f90:249-595)
    def integrate(self, t: float, tout: float, y: np.ndarray):
        """Returns (y(tout), tout, iflag); iflag 2 on success, 3 tolerances raised, 4 too many steps,
        5 too many steps and the problem appears stiff (the reference's codes)."""
        fouru = 4.0 * _EPS
        iflag = self.iflag
        if t == tout or self.relerr < 0 or self.abserr < 0:
            raise ValueError("AdamsIntegrator: bad arguments")
        eps = max(self.relerr, self.abserr)
        isn = 1 if iflag > 0 else -1
        iflag = abs(iflag)
        if iflag != 1 and t != self.told:
            raise ValueError("AdamsIntegrator: t changed between calls")
        dl = tout - t
        absdel = abs(dl)
        tend = tout if isn < 0 else t + 10.0 * dl
        nostep = kle4 = 0
        stiff = False
        releps, abseps = self.relerr / eps, self.abserr / eps
        y = np.array(y, dtype=np.float64, copy=True)
        if iflag == 1 or self.isnold < 0 or self.delsgn * dl <= 0.0:
            self.start = True
            self.x = t
            self.yy[:] = y
            self.delsgn = 1.0 if dl >= 0 else -1.0
            self.h = np.copysign(max(abs(tout - self.x), fouru * abs(self.x)), tout - self.x)
        while True:
            if absdel <= abs(self.x - t):
                y = self._intrp(tout)
                self.iflag = 2
                self.told = tout
                self.isnold = isn
                return y, tout, 2
            if isn <= 0 and abs(tout - self.x) < fouru * abs(self.x):
                h = tout - self.x
                yp = self._f(self.x, self.yy)
                self.iflag = 2
                self.told = tout
                self.isnold = isn
                return self.yy + h * yp, tout, 2
            if self.MAXNUM <= nostep:
                code = isn * (5 if stiff else 4)
                self.iflag = code
                self.told = self.x
                self.isnold = 1
                return self.yy.copy(), self.x, code
            self.h = np.copysign(min(abs(self.h), abs(tend - self.x)), self.h)
            self.wt[:] = releps * np.abs(self.yy) + abseps
            crash, eps = self._step(eps)
            if crash:
                self.relerr, self.abserr = eps * releps, eps * abseps
                self.iflag = isn * 3
                self.told = self.x
                self.isnold = 1
                return self.yy.copy(), self.x, isn * 3
            nostep += 1
            self.steps += 1
            kle4 += 1
            if self.kold > 4:
                kle4 = 0
            if kle4 >= 50:
                stiff = True

    # ------------------------------------------------------------------ step (src/adams_ode.f90:597-1230)
    def _step(self, eps):
        twou = 2.0 * _EPS
        fouru = 2.0 * twou
        x, y, wt, phi, psi = self.x, self.yy, self.wt, self.phi, self.psi
        alpha, beta, sig, v, w, g = self.alpha, self.beta, self.sig, self.v, self.w, self.g
        h = self.h
        if abs(h) < fouru * abs(x):
            self.h = np.copysign(fouru * abs(x), h)
            return True, eps
        p5eps = 0.5 * eps
        rnd = twou * float(np.sqrt(np.sum((y / wt) ** 2)))
        if p5eps < rnd:
            return True, 2.0 * rnd * (1.0 + fouru)
        g[1], g[2], sig[1] = 1.0, 0.5, 1.0
        if self.start:
            yp = self._f(x, y)
            phi[1] = yp
            phi[2] = 0.0
            total = float(np.sqrt(np.sum((yp / wt) ** 2)))
            absh = abs(h)
            if eps < 16.0 * total * h * h:
                absh = 0.25 * np.sqrt(eps / total)
            h = np.copysign(max(absh, fouru * abs(x)), h)
            self.hold = 0.0
            self.k, self.kold = 1, 0
            self.start = False
            self.phase1 = True
            self.nornd = True
            if p5eps <= 100.0 * rnd:
                self.nornd = False
                phi[15] = 0.0
        ifail = 0
        k, kold, ns = self.k, self.kold, self.ns
        while True:
            kp1, kp2, km1, km2 = k + 1, k + 2, k - 1, k - 2
            if h != self.hold:
                ns = 0
            if ns <= kold:
                ns += 1
            nsp1 = ns + 1
            if ns <= k:
                # coefficients that change with the step size
                beta[ns] = 1.0
                alpha[ns] = 1.0 / ns
                temp1 = h * ns
                sig[nsp1] = 1.0
                for i in range(nsp1, k + 1):
                    temp2 = psi[i - 1]
                    psi[i - 1] = temp1
                    beta[i] = beta[i - 1] * psi[i - 1] / temp2
                    temp1 = temp2 + h
                    alpha[i] = h / temp1
                    sig[i + 1] = i * alpha[i] * sig[i]
                psi[k] = temp1
                if ns <= 1:
                    for iq in range(1, k + 1):
                        v[iq] = 1.0 / (iq * (iq + 1))
                        w[iq] = v[iq]
                else:
                    if kold < k:
                        v[k] = 1.0 / (k * kp1)
                        for j in range(1, ns - 1):
                            i = k - j
                            v[i] = v[i] - alpha[j + 1] * v[i + 1]
                    for iq in range(1, kp1 - ns + 1):
                        v[iq] = v[iq] - alpha[ns] * v[iq + 1]
                        w[iq] = v[iq]
                    g[nsp1] = w[1]
                for i in range(ns + 2, kp1 + 1):
                    for iq in range(1, kp2 - i + 1):
                        w[iq] = w[iq] - alpha[i - 1] * w[iq + 1]
                    g[i] = w[1]
            for i in range(nsp1, k + 1):
                phi[i] *= beta[i]
            phi[kp2] = phi[kp1]
            phi[kp1] = 0.0
            p = np.zeros(self.neq)
            for j in range(1, k + 1):
                i = kp1 - j
                p += phi[i] * g[i]
                phi[i] += phi[i + 1]
            if not self.nornd:
                tau = h * p - phi[15]
                p = y + tau
                phi[16] = (p - y) - tau
            else:
                p = y + h * p
            xold = x
            x = x + h
            absh = abs(h)
            yp = self._f(x, p)
            # error estimates at orders k-2, k-1, k and the order to use next
            erkm2 = erkm1 = 0.0
            if km2 > 0:
                erkm2 = float(np.sum(((phi[km1] + yp - phi[1]) / wt) ** 2))
            if km2 >= 0:
                erkm1 = float(np.sum(((phi[k] + yp - phi[1]) / wt) ** 2))
            erk = float(np.sum(((yp - phi[1]) / wt) ** 2))
            if km2 > 0:
                erkm2 = absh * sig[km1] * _GSTR[km2] * np.sqrt(erkm2)
            if km2 >= 0:
                erkm1 = absh * sig[k] * _GSTR[km1] * np.sqrt(erkm1)
            err = absh * np.sqrt(erk) * (g[k] - g[kp1])
            erk = absh * np.sqrt(erk) * sig[kp1] * _GSTR[k]
            knew = k
            if km2 > 0:
                if max(erkm1, erkm2) <= erk:
                    knew = km1
            elif km2 == 0:
                if erkm1 <= 0.5 * erk:
                    knew = km1
            if not np.isfinite(err):
                raise FloatingPointError("AdamsIntegrator: the error estimate is not finite")
            if err <= eps:
                break
            # unsuccessful step: restore x, phi, psi and halve the step (or more)
            self.phase1 = False
            x = xold
            for i in range(1, k + 1):
                phi[i] = (phi[i] - phi[i + 1]) / beta[i]
            for i in range(2, k + 1):
                psi[i - 1] = psi[i] - h
            ifail += 1
            temp2 = 0.5
            if ifail > 3 and p5eps < 0.25 * erk:
                temp2 = np.sqrt(p5eps / erk)
            if ifail >= 3:
                knew = 1
            h = temp2 * h
            k = knew
            if abs(h) < fouru * abs(x):
                self.h = np.copysign(fouru * abs(x), h)
                self.x, self.k, self.kold, self.ns = x, k, kold, ns
                return True, eps + eps
        # successful step: correct, evaluate, update the differences
        kold = k
        self.hold = h
        if not self.nornd:
            rho = h * g[kp1] * (yp - phi[1]) - phi[16]
            ynew = p + rho
            phi[15] = (ynew - p) - rho
        else:
            ynew = p + h * g[kp1] * (yp - phi[1])
        y[:] = ynew
        yp = self._f(x, y)
        phi[kp1] = yp - phi[1]
        phi[kp2] = phi[kp1] - phi[kp2]
        for i in range(1, k + 1):
            phi[i] += phi[kp1]
        # the order for the next step
        erkp1 = 0.0
        if knew == km1 or k == 12:
            self.phase1 = False
        if self.phase1:
            k = kp1
            erk = erkp1
        elif knew == km1:
            k = km1
            erk = erkm1
        elif kp1 <= ns:
            erkp1 = absh * _GSTR[kp1] * np.sqrt(float(np.sum((phi[kp2] / wt) ** 2)))
            if k == 1:
                if erkp1 < 0.5 * erk:
                    k = kp1
                    erk = erkp1
            elif erkm1 <= min(erk, erkp1):
                k = km1
                erk = erkm1
            elif erkp1 < erk and k < 12:
                k = kp1
                erk = erkp1
        # the step size for the next step
        hnew = h + h
        if not self.phase1 and p5eps < erk * _TWO[k + 1]:
            hnew = h
            if p5eps < erk:
                r = (p5eps / erk) ** (1.0 / (k + 1))
                hnew = absh * max(0.5, min(0.9, r))
                hnew = np.copysign(max(hnew, fouru * abs(x)), h)
        self.h = hnew
        self.x, self.k, self.kold, self.ns = x, k, kold, ns
        return False, eps

    # ------------------------------------------------------------------ intrp (src/adams_ode.f90:1232-1357)
    def _intrp(self, xout):
        hi = xout - self.x
        ki = self.kold + 1
        w = np.zeros(14)
        gg = np.zeros(14)
        rho = np.zeros(14)
        for i in range(1, ki + 1):
            w[i] = 1.0 / i
        gg[1] = rho[1] = 1.0
        term = 0.0
        for j in range(2, ki + 1):
            psijm1 = self.psi[j - 1]
            gamma = (hi + term) / psijm1
            eta = hi / psijm1
            for i in range(1, ki + 2 - j):
                w[i] = gamma * w[i] - eta * w[i + 1]
            gg[j] = w[1]
            rho[j] = gamma * rho[j - 1]
            term = psijm1
        yout = np.zeros(self.neq)
        ypout = np.zeros(self.neq)
        for j in range(1, ki + 1):
            i = ki + 1 - j
            yout += gg[i] * self.phi[i]
            ypout += rho[i] * self.phi[i]
        self.ypout[:] = ypout
        return self.yy + hi * yout


@dataclass
class OdeFlowResult:
    steps: list = field(default_factory=list)  # (step, s, E0, E0 + MBPT2, |MBPT2|)
    evaluations: int = 0

    @property
    def E0(self) -> float:
        return self.steps[-1][2] if self.steps else float("nan")


def decouple_hamiltonian(eng: Engine, H0: np.ndarray, generator: str = "white", ds: float = 0.1,
                         max_steps: int = 10000, conv_crit: float = 1e-6, relerr: float = 1e-6, abserr: float = 1e-6,
                         s_max: float | None = None, ops: dict | None = None, prefix: str | None = None,
                         output_dir: str = ".", derivative=None) -> OdeFlowResult:
    """decouple_hamiltonian (src/IMSRG_ODE.f90:9-178) for one operator: the vectorized H(s) is
    advanced by the Adams integrator over intervals ds = 0.1 with relerr = abserr = 1e-6 until
    |MBPT2| < 1e-6 (or max_steps intervals, or s_max).  dH/ds = vectorize([eta(H), H]) is the
    device's (dHds, :416-463).  With prefix set, the per-interval line is written to
    <output_dir>/<prefix>_0bflow.dat ('(I6,4(e17.9))' for the first line, '(I6,4(e15.7))' after,
    as the reference writes them).  `derivative(s, y) -> y'` replaces the device derivative
    (used to drive the same integrator with another evaluator)."""
    gens = {"white": eng.build_gs_white, "atan": eng.build_gs_atan, "w2": eng.build_gs_w2}
    if generator not in gens:
        raise ValueError(f"generator must be one of {sorted(gens)}")
    build = gens[generator]
    HS, ETA, DH = eng.new_op(1, H0), eng.new_op(-1), eng.new_op(1)
    neq = eng.neq

    def device_derivative(s, y):
        HS.upload(eng.repackage(y, 1))
        build(HS, ETA)
        eng.commutator(ETA, HS, DH)
        return eng.vectorize(DH.download())

    f = derivative or device_derivative
    integ = AdamsIntegrator(f, neq, relerr, abserr)
    res = OdeFlowResult()
    lines = []
    y = eng.vectorize(np.asarray(H0, dtype=np.float64))
    s = 0.0
    H = np.asarray(H0, dtype=np.float64)
    e2 = eng.mbpt2(HS)
    res.steps.append((0, s, float(H[0]), float(H[0]) + e2, abs(e2)))
    lines.append(f"{0:6d}" + "".join(_e_fmt(x, 17, 9) for x in (s, H[0], H[0] + e2, abs(e2))))
    steps = 0
    crit = abs(e2)
    while steps < max_steps and crit >= conv_crit:
        if s_max is not None and s >= s_max - 1e-12:
            break
        y, s, iflag = integ.integrate(s, s + ds, y)
        if iflag != 2:
            raise RuntimeError(f"Adams integration stopped with iflag {iflag} at s={s}")
        H = eng.repackage(y, 1)
        HS.upload(H)
        steps += 1
        e2 = eng.mbpt2(HS)
        crit = abs(e2)
        res.steps.append((steps, s, float(H[0]), float(H[0]) + e2, crit))
        lines.append(f"{steps:6d}" + "".join(_e_fmt(x, 15, 7) for x in (s, H[0], H[0] + e2, crit)))
    res.evaluations = integ.evaluations
    if prefix is not None:
        with open(os.path.join(output_dir, f"{prefix.strip()}_0bflow.dat"), "w") as fh:
            fh.write("\n".join(lines) + "\n")
    if ops is not None:
        ops.update(HS=HS)
    return res


def _e_fmt(x: float, width: int, digits: int) -> str:
    """Fortran's e<width>.<digits> edit descriptor: 0.ddd...E+xx, right-justified."""
    x = float(x)
    if x == 0.0:
        s = "0." + "0" * digits + "E+00"
        return f"{s:>{width}}"
    exp = int(np.floor(np.log10(abs(x)))) + 1
    v = round(abs(x) / 10.0 ** exp, digits)
    if v >= 1.0:
        v /= 10.0
        exp += 1
    s = f"{'-' if x < 0 else ''}0.{int(round(v * 10 ** digits)):0{digits}d}E{'+' if exp >= 0 else '-'}{abs(exp):02d}"
    return f"{s:>{width}}"
