"""Solver settings of the measured workloads (IMS LINEAR and NONLINEAR blocks).

C2 (1000x1000x10 confined steady state): PCG + ILU0, INNER_DVCLOSE 1e-6 m,
INNER_RCLOSE 1e-2 m3/d (infinity norm), OUTER_DVCLOSE 1e-6 m.
C1 (100x100x1): the configuration's INNER_DVCLOSE 1e-8, INNER_RCLOSE 1e-6.
"""
C1_IMS = dict(dvclose=1e-8, rclose=1e-6, iter1=1000, ilinmeth=1)
C1_OUTER = dict(dvclose=1e-8, mxiter=10)
C2_IMS = dict(dvclose=1e-6, rclose=1e-2, iter1=20000, ilinmeth=1)
C2_OUTER = dict(dvclose=1e-6, mxiter=10)
