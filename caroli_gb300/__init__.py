"""caroli_gb300 — GB300-native (sm_103a) nested-dissection transport of caroli.

The hot path (front assembly, pivot-block elimination, Schur updates, root solve and Caroli trace)
runs in ``libcaroli_gb300.so`` (``csrc/``), reached through the C ABI of
``include/caroli_gb300.h``; this package is the host face that mirrors caroli's Rust API:
``NestedTwoTerminal`` (transmissions, precisions, gradients, scattering states, bond currents,
densities, transmission eigenvalues, scattering matrix), ``NestedMultiTerminal`` (T_pq, sector
transmissions, scattering states, scattering matrix), lead self-energies, models and disorder.
"""
from .lattice import Lattice, Region, Site
from .leads import GreenError, LeadSolver, broadening, gamma_root
from .model import BhzParams, Model, OnSiteMap, SparseMatrix, bhz, bhz_exchange, bhz_spin, cubic, graphene, square
from .nested import LeadSelfEnergies, NestedTwoTerminal, solve_systems
from .precision import Precision, PrecisionOptions, PrecisionReport, checked
from .states import BondCurrent, ScatteringStates
from .multi import AttachedLead, Interface, MultiSelfEnergies, NestedMultiTerminal, attach_leads, lead_voltages
from .nested import ModeSelfEnergies
from .smatrix import SMatrix
from .system import System, build_system

__all__ = [
    "Lattice", "Region", "Site", "GreenError", "LeadSolver", "broadening", "gamma_root", "BhzParams", "Model",
    "OnSiteMap", "SparseMatrix", "bhz", "bhz_exchange", "bhz_spin", "cubic", "graphene", "square",
    "LeadSelfEnergies", "NestedTwoTerminal", "solve_systems", "Precision", "PrecisionOptions", "PrecisionReport", "checked",
    "System", "build_system", "BondCurrent", "ScatteringStates", "AttachedLead", "Interface",
    "NestedMultiTerminal", "attach_leads", "lead_voltages", "MultiSelfEnergies", "ModeSelfEnergies", "SMatrix",
]
