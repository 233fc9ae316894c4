"""Builds and imports the reference Florence package (pure-Python assembly path).

Test infrastructure only: used to generate the golden fixtures in this folder.
It runs where a checkout of the reference is available (its root directory
named by the environment variable ``FLORENCE_REFERENCE``); it never runs on the
GPU machine and nothing in the product imports it.

What it does (the reference cannot be built as shipped: its native element
kernels need the third-party Fastor headers, CBLAS and x86 intrinsics):

1. copies ``$FLORENCE_REFERENCE/Florence`` to ``baseline/_ref/Florence`` (git-ignored);
2. compiles the ten Fastor-free Cython modules of the reference from their own
   sources (tensor helpers, Jacobi/Bernstein bases, geometric stiffness, Voigt
   B-matrix filler, sparse/RHS assembly helpers and ``ComputeSparsityPattern``);
3. writes stub modules for the seven Fastor-only modules (``_KinematicMeasures_``,
   ``_ConstitutiveStiffnessDF_`` ...), so that ``import Florence`` succeeds and
   the reference falls back to its own numpy element path
   (``DisplacementFormulation.GetLocalStiffness``,
   Florence/VariationalPrinciple/DisplacementFormulation.py:110-188);
4. adds numpy-2 aliases for names the reference still uses (``np.in1d`` ...).
"""
import os
import shutil
import subprocess
import sys
import sysconfig

REF_ROOT = os.environ.get("FLORENCE_REFERENCE", "")  # root of the read-only reference checkout
REF_SRC = os.path.join(REF_ROOT, "Florence")
REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
HARNESS_ROOT = os.path.join(REPO, "baseline", "_ref")
PKG = os.path.join(HARNESS_ROOT, "Florence")

# (pyx relative to the package, extra include dirs relative to the package, output dir relative to the package)
CYTHON_MODULES = [
    ("Tensor/Numeric.pyx", ["Tensor"], "Tensor", ["Tensor/_Numeric.cpp"]),
    ("Tensor/LinAlg.pyx", ["Tensor"], "Tensor", ["Tensor/_LinAlg.cpp"]),
    ("FunctionSpace/JacobiPolynomials/JacobiPolynomials.pyx", [], "FunctionSpace/JacobiPolynomials", []),
    ("FunctionSpace/OneDimensional/_OneD/LineBP.pyx", ["FunctionSpace/OneDimensional/_OneD", "Tensor"],
     "FunctionSpace/OneDimensional", []),
    ("VariationalPrinciple/_GeometricStiffness_/_GeometricStiffness_.pyx", ["VariationalPrinciple/_GeometricStiffness_"],
     "VariationalPrinciple", []),
    ("VariationalPrinciple/_ConstitutiveStiffness_/DisplacementApproachIndices.pyx", [], "VariationalPrinciple", []),
    ("VariationalPrinciple/_ConstitutiveStiffness_/DisplacementPotentialApproachIndices.pyx", [],
     "VariationalPrinciple", []),
    ("FiniteElements/Assembly/_Assembly_/SparseAssemblyNative.pyx", ["FiniteElements/Assembly/_Assembly_"],
     "FiniteElements/Assembly", []),
    ("FiniteElements/Assembly/_Assembly_/RHSAssemblyNative.pyx", ["FiniteElements/Assembly/_Assembly_"],
     "FiniteElements/Assembly", []),
    ("FiniteElements/Assembly/_Assembly_/ComputeSparsityPattern.pyx", ["FiniteElements/Assembly/_Assembly_"],
     "FiniteElements/Assembly", []),
]

STUBS = {
    "FiniteElements/LocalAssembly/_KinematicMeasures_.py": ["_KinematicMeasures_"],
    "VariationalPrinciple/_ConstitutiveStiffnessDF_.py": ["__ConstitutiveStiffnessIntegrandDF__"],
    "VariationalPrinciple/_ConstitutiveStiffnessDPF_.py": ["__ConstitutiveStiffnessIntegrandDPF__"],
    "VariationalPrinciple/_ConstitutiveStiffnessLaplacian_.py": ["__ConstitutiveStiffnessIntegrandLaplacian__"],
    "VariationalPrinciple/_TractionDF_.py": ["__TractionIntegrandDF__"],
    "VariationalPrinciple/_TractionDPF_.py": ["__TractionIntegrandDPF__"],
    "VariationalPrinciple/_MassIntegrand_.py": ["__MassIntegrand__", "__ConstantMassIntegrand__",
                                                "__TotalConstantMassIntegrand__"],
}


def _compile(pyx, incs, outdir, extra_cpp):
    import numpy as np
    name = os.path.splitext(os.path.basename(pyx))[0]
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    target = os.path.join(PKG, outdir, name + suffix)
    if os.path.exists(target):
        return
    src = os.path.join(PKG, pyx)
    cpp = os.path.splitext(src)[0] + ".cpp"
    subprocess.check_call([sys.executable, "-m", "cython", "--cplus", "-3", "-X", "language_level=3", src, "-o", cpp])
    cmd = ["g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
           "-I" + sysconfig.get_paths()["include"], "-I" + np.get_include()]
    for d in incs:
        cmd.append("-I" + os.path.join(PKG, d))
    cmd += [cpp] + [os.path.join(PKG, e) for e in extra_cpp] + ["-o", target]
    subprocess.check_call(cmd)


def build():
    """Create the patched copy and compile what can be compiled (idempotent)."""
    if not os.path.isdir(REF_SRC) and not os.path.isdir(PKG):
        raise RuntimeError("reference checkout not found at %r (set FLORENCE_REFERENCE to its root)" % REF_SRC)
    if not os.path.isdir(PKG):
        os.makedirs(HARNESS_ROOT, exist_ok=True)
        shutil.copytree(REF_SRC, PKG)
    for pyx, incs, outdir, extra in CYTHON_MODULES:
        _compile(pyx, incs, outdir, extra)
    for rel, names in STUBS.items():
        path = os.path.join(PKG, rel)
        if os.path.exists(path):
            continue
        with open(path, "w") as f:
            f.write("# stub: the native module needs Fastor, which is not available\n")
            for n in names:
                f.write("def %s(*args, **kwargs):\n    raise NotImplementedError('%s needs Fastor')\n" % (n, n))


def _numpy2_aliases():
    import numpy as np
    aliases = {"in1d": np.isin, "NAN": np.nan, "NaN": np.nan, "Inf": np.inf, "product": np.prod,
               "cumproduct": np.cumprod, "alltrue": np.all, "sometrue": np.any, "row_stack": np.vstack,
               "float_": np.float64, "int_": np.int64,
               "asfarray": lambda a, dtype=np.float64: np.asarray(a, dtype=dtype)}
    for k, v in aliases.items():
        if not hasattr(np, k):
            setattr(np, k, v)


def import_florence():
    """Build if needed, then import the reference package and return it."""
    build()
    _numpy2_aliases()
    if HARNESS_ROOT not in sys.path:
        sys.path.insert(0, HARNESS_ROOT)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import Florence  # noqa: F401
    import numpy as np
    # high-order tet/tri node generation passes 1-element arrays where scalars are expected
    from Florence.FunctionSpace.ThreeDimensional.Tet import hpNodal as tet_hp
    from Florence.FunctionSpace.TwoDimensional.Tri import hpNodal as tri_hp
    for mod, fname in ((tet_hp, "GradNormalisedJacobiTet"), (tri_hp, "GradNormalisedJacobiTri")):
        if hasattr(mod, fname) and not getattr(getattr(mod, fname), "_wrapped", False):
            orig = getattr(mod, fname)

            def wrapped(*args, _orig=orig):
                args = list(args)
                for i, a in enumerate(args):
                    if isinstance(a, np.ndarray):
                        args[i] = np.asarray(a, np.float64).ravel()
                return _orig(*args)
            wrapped._wrapped = True
            setattr(mod, fname, wrapped)
    return Florence
