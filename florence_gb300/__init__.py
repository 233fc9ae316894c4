"""florence_gb300 -- GB300-native (sm_103a) low-level finite-element assembly for Florence's
displacement formulation: fused FP64 tangent + residual kernels, a device-built CSR pattern
with the reference's element-to-nonzero maps, a matrix-free explicit internal force, lumped and
consistent mass, external forces, the displacement-potential (electromechanics) assembly and
high-order tet meshing, behind Florence's own low-level assembly interface.

The CUDA library (libflorence_gb300.so, built in-tree) is required: nothing here falls back to
the CPU.
"""
from . import _native
from .assembly import (AssembleBodyForces, AssembleExternalTractionForces, ComputeSparsityPattern, DeviceAssembler, _LowLevelAssemblyDF__AnisotropicMooneyRivlin_1_,
                       _LowLevelAssemblyDF__LinearElastic_,
                       _LowLevelAssemblyDF__MooneyRivlin_, _LowLevelAssemblyDF__NearlyIncompressibleMooneyRivlin_,
                       _LowLevelAssemblyDF__NeoHookean_, _LowLevelAssemblyExplicit_DF_DPF_,
                       __TotalConstantMassIntegrand__, arithmetic, device_sparsity, fp32_peak_gflops, fp64_peak_gflops,
                       get_arithmetic, install, material_params, release_device_meshes, release_host_buffers, set_arithmetic,
                       set_tensor_core_tiling)
from .electromechanics import (DPFAssembler, _LowLevelAssemblyDPF__IsotropicElectroMechanics_0_,
                               _LowLevelAssemblyDPF__IsotropicElectroMechanics_101_,
                               _LowLevelAssemblyDPF__IsotropicElectroMechanics_105_,
                               _LowLevelAssemblyDPF__IsotropicElectroMechanics_106_,
                               _LowLevelAssemblyDPF__IsotropicElectroMechanics_108_,
                               _LowLevelAssemblyDPF__Piezoelectric_100_, _LowLevelAssemblyDPF__SteinmannModel_)

__all__ = ["AssembleBodyForces", "AssembleExternalTractionForces", "ComputeSparsityPattern", "DeviceAssembler", "DPFAssembler",
           "_LowLevelAssemblyDPF__IsotropicElectroMechanics_108_", "_LowLevelAssemblyDPF__IsotropicElectroMechanics_101_",
           "_LowLevelAssemblyDPF__IsotropicElectroMechanics_0_", "_LowLevelAssemblyDPF__IsotropicElectroMechanics_106_",
           "_LowLevelAssemblyDPF__IsotropicElectroMechanics_105_", "_LowLevelAssemblyDPF__SteinmannModel_",
           "_LowLevelAssemblyDPF__Piezoelectric_100_",
           "_LowLevelAssemblyDF__NeoHookean_",
           "_LowLevelAssemblyDF__AnisotropicMooneyRivlin_1_",
           "_LowLevelAssemblyDF__MooneyRivlin_", "_LowLevelAssemblyDF__NearlyIncompressibleMooneyRivlin_",
           "_LowLevelAssemblyDF__LinearElastic_", "_LowLevelAssemblyExplicit_DF_DPF_",
           "__TotalConstantMassIntegrand__", "arithmetic", "device_sparsity", "fp32_peak_gflops", "fp64_peak_gflops", "get_arithmetic",
           "install", "material_params", "release_device_meshes", "release_host_buffers", "set_arithmetic",
           "set_tensor_core_tiling"]
