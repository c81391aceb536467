"""Solver settings of the measured workloads (IMS LINEAR and NONLINEAR blocks).

C2 (1000x1000x10 confined steady state): PCG + ILU0, INNER_DVCLOSE 1e-4 m,
INNER_RCLOSE 1e-5 m3/d (infinity norm), OUTER_DVCLOSE 1e-4 m.  The tight
RCLOSE, not the last step size, bounds the head error (about 1e-6 m in FP64
against a solve converged far below it, a few 1e-6 m in the mixed form), so
the FP64 and mixed heads agree within 0.1 x INNER_DVCLOSE.
C1 (100x100x1): the configuration's INNER_DVCLOSE 1e-8, INNER_RCLOSE 1e-6.
C3 (500x500x5 convertible, NEWTON, transient): BiCGSTAB + ILU0 with
INNER_DVCLOSE 1e-4 m and INNER_RCLOSE 1e-2 m3/d, the MODERATE preset's DBD
under-relaxation (sln_setouter NumericalSolution.f90:2644-2655: theta 0.9,
kappa 1e-4, gamma 0) with OUTER_DVCLOSE 1e-5 m and OUTER_MAXIMUM 100; ten
stress periods of 10 d, each 10 steps with TSMULT 1.2.
"""
C1_IMS = dict(dvclose=1e-8, rclose=1e-6, iter1=1000, ilinmeth=1)
C1_OUTER = dict(dvclose=1e-8, mxiter=10)
C2_IMS = dict(dvclose=1e-4, rclose=1e-5, iter1=20000, ilinmeth=1)
C2_OUTER = dict(dvclose=1e-4, mxiter=10)
# C4 (256-member ensemble of confined steady-state DIS grids): PCG + ILU0
# with the C2 closures, every member to its own closure.
C4_IMS = dict(dvclose=1e-6, rclose=1e-4, iter1=20000, ilinmeth=1)
C3_IMS = dict(dvclose=1e-4, rclose=1e-2, iter1=500, ilinmeth=2)
C3_OUTER = dict(dvclose=1e-5, mxiter=100, nonmeth=3, theta=0.9, akappa=1e-4, gamma=0.0,
                amomentum=0.0)
C3_PERIOD = dict(nper=10, perlen=10.0, nstp=10, tsmult=1.2)


def step_lengths(perlen: float, nstp: int, tsmult: float, totim: float = 0.0) -> list:
    """TDIS time-step lengths of one stress period that starts at simulation
    time `totim` (tdis_set_delt, src/Timing/tdis.f90:247-268): the first step
    perlen*(1-tsmult)/(1-tsmult**nstp) (perlen/nstp when tsmult is 1), each
    later step tsmult times the previous, and the last one whatever reaches
    the end of the period exactly."""
    topertim = totim
    out = []
    delt = 0.0
    for kstp in range(1, nstp + 1):
        if kstp == 1:
            if tsmult != 1.0:
                delt = perlen * (1.0 - tsmult) / (1.0 - tsmult ** nstp)
            else:
                delt = perlen / float(nstp)
        elif kstp == nstp:
            delt = topertim + perlen - totim
        else:
            delt = tsmult * delt
        out.append(delt)
        totim = totim + delt
    return out
