"""Solver settings of the measured workloads (IMS LINEAR and NONLINEAR blocks).

C2 (1000x1000x10 confined steady state): PCG + ILU0, INNER_DVCLOSE 1e-4 m,
INNER_RCLOSE 1e-5 m3/d (infinity norm), OUTER_DVCLOSE 1e-4 m.  The tight
RCLOSE, not the last step size, bounds the head error (about 1e-6 m in FP64
against a solve converged far below it, a few 1e-6 m in the mixed form), so
the FP64 and mixed heads agree within 0.1 x INNER_DVCLOSE.
C1 (100x100x1): the configuration's INNER_DVCLOSE 1e-8, INNER_RCLOSE 1e-6.
"""
C1_IMS = dict(dvclose=1e-8, rclose=1e-6, iter1=1000, ilinmeth=1)
C1_OUTER = dict(dvclose=1e-8, mxiter=10)
C2_IMS = dict(dvclose=1e-4, rclose=1e-5, iter1=20000, ilinmeth=1)
C2_OUTER = dict(dvclose=1e-4, mxiter=10)
# C4 (256-member ensemble of confined steady-state DIS grids): PCG + ILU0
# with the C2 closures, every member to its own closure.
C4_IMS = dict(dvclose=1e-6, rclose=1e-4, iter1=20000, ilinmeth=1)
