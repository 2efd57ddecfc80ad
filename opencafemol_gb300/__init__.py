"""GB300-native force-and-integrate engine for OpenCafeMol's coarse-grained
protein force field (harmonic bonds, Go 10-12 contacts, flexible-local
angles and dihedrals, AICG2+ Gaussian bonds and dihedrals, excluded volume,
Debye-Hueckel, HPS Lennard-Jones, Weeks-Chandler-Andersen, capped Go) with
a Langevin integrator and a local energy minimiser, behind the C ABI in
include/ocm.h.
"""
from ._lib import LIB_PATH, OCMError, device_count, lib
from .engine import ALL_GROUPS, Batch, Context, LocalEnergyMinimizer
from .forcefield import (AMINO_ACIDS, CappedGoContactForceFieldGenerator, DebyeHuckelForceFieldGenerator,
                         ExcludedVolumeForceFieldGenerator,
                         FlexibleLocalAngleForceFieldGenerator,
                         FlexibleLocalDihedralForceFieldGenerator, GaussianBondForceFieldGenerator,
                         GaussianDihedralForceFieldGenerator, GoContactForceFieldGenerator,
                         HarmonicBondForceFieldGenerator, LangevinIntegrator,
                         LangevinIntegratorGenerator, LennardJonesAttractiveForceFieldGenerator,
                         LennardJonesRepulsiveForceFieldGenerator, System, SystemGenerator,
                         Topology, UniformLennardJonesAttractiveForceFieldGenerator,
                         UniformWeeksChandlerAndersenForceFieldGenerator,
                         WeeksChandlerAndersenForceFieldGenerator, cutoff_ratio_for,
                         fla_second_derivative_table, fla_spline_table, fld_fourier_table,
                         fld_table_keys)

__all__ = [
    "LIB_PATH", "OCMError", "device_count", "lib", "ALL_GROUPS", "Batch", "Context", "LocalEnergyMinimizer",
    "AMINO_ACIDS", "DebyeHuckelForceFieldGenerator", "ExcludedVolumeForceFieldGenerator",
    "FlexibleLocalAngleForceFieldGenerator", "FlexibleLocalDihedralForceFieldGenerator",
    "GaussianBondForceFieldGenerator", "GaussianDihedralForceFieldGenerator",
    "GoContactForceFieldGenerator", "HarmonicBondForceFieldGenerator", "LangevinIntegrator",
    "LangevinIntegratorGenerator", "LennardJonesAttractiveForceFieldGenerator",
    "LennardJonesRepulsiveForceFieldGenerator", "System", "SystemGenerator", "Topology",
    "cutoff_ratio_for", "fla_second_derivative_table", "fla_spline_table", "fld_fourier_table",
    "fld_table_keys", "WeeksChandlerAndersenForceFieldGenerator",
    "UniformWeeksChandlerAndersenForceFieldGenerator", "UniformLennardJonesAttractiveForceFieldGenerator",
    "CappedGoContactForceFieldGenerator",
]
