"""CPU check that install() wires the GPU callables into the reference's own dispatcher.

Runs only where the reference package is importable (the container that builds the golden
fixtures); the GPU parity of the callables themselves is in test_gpu_assembly.py.
"""
import os
import sys

import pytest

from conftest import ROOT

HARNESS = os.path.join(ROOT, "baseline", "_ref", "Florence")
REFERENCE = os.environ.get("FLORENCE_REFERENCE", "")  # root of a reference checkout, where there is one


@pytest.mark.skipif(not os.path.isdir(HARNESS) or not REFERENCE or not os.path.isdir(REFERENCE),
                    reason="reference package not available here")
def test_install_registers_callables_in_reference_namespaces():
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import florence_harness
    F = florence_harness.import_florence()
    import florence_gb300
    ll = florence_gb300.install(F)
    from Florence.FiniteElements.Assembly import _LowLevelAssembly_ as mod
    assert mod is ll
    for mat in ("NeoHookean", "MooneyRivlin", "NearlyIncompressibleMooneyRivlin", "LinearElastic",
                "AnisotropicMooneyRivlin_1"):
        name = "_LowLevelAssemblyDF__" + mat + "_"
        assert getattr(mod, name) is getattr(florence_gb300, name)
    assert mod._LowLevelAssemblyExplicit_DF_DPF_ is florence_gb300._LowLevelAssemblyExplicit_DF_DPF_
    # the electromechanics (displacement-potential) entry, found by the dispatcher's "DPF" prefix
    assert (mod._LowLevelAssemblyDPF__IsotropicElectroMechanics_108_
            is florence_gb300._LowLevelAssemblyDPF__IsotropicElectroMechanics_108_)
    em = F.IsotropicElectroMechanics_108(3, mu1=0.5, mu2=0.3, lamb=10.0, eps_2=2.0)
    assert ("_LowLevelAssemblyDPF__" + type(em).__name__ + "_") in vars(mod)
    for em_name in ("IsotropicElectroMechanics_101", "IsotropicElectroMechanics_0", "IsotropicElectroMechanics_106",
                    "IsotropicElectroMechanics_105", "SteinmannModel", "Piezoelectric_100"):
        name = "_LowLevelAssemblyDPF__" + em_name + "_"
        assert getattr(mod, name) is getattr(florence_gb300, name)
    from Florence.FiniteElements.Assembly.ComputeSparsityPattern import ComputeSparsityPattern
    assert ComputeSparsityPattern is florence_gb300.ComputeSparsityPattern
    # the dispatcher's own name lookup now finds the GPU callable
    mat = F.NeoHookean(3, mu=1.0, lamb=10.0)
    assert ("_LowLevelAssemblyDF__" + type(mat).__name__ + "_") in vars(mod)
