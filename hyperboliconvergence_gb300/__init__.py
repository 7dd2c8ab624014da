"""GB300-native residual-and-timestep path of a 2D finite-volume Euler solver.

Least-squares gradients, MUSCL reconstruction with slope limiters, Roe / SLAU /
AUSM+up face fluxes, face-to-cell accumulation, global or local timestep and
the SSP Runge-Kutta update, as hand-written sm_103a CUDA behind the C ABI in
include/hc.h.
"""
from ._capi import HCError, load
from .solver import Mesh, Solver

__all__ = ["HCError", "Mesh", "Solver", "load"]
