"""Import modules of the reference checkout (fixture generation only).

The reference's Python package needs pandas, pandapower and numba, none of which this
project's environment has. The modules whose functions the fixtures call use them only for
type annotations, for ``numba.njit`` / ``prange`` (which change the speed, not the
arithmetic, of a loop) and, in the transformer model, for one ``pandas.MultiIndex`` lookup.
``install()`` puts minimal stand-ins for the three packages into ``sys.modules`` and the
reference checkout on ``sys.path``, so ``import p3s.<module>`` then loads the reference's own
source unchanged.
"""

import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import build as ob  # noqa: E402


class _Anything:
    """Stand-in for any name a stubbed package exports (classes used in annotations,
    exception types, decorators): callable, subclassable, and every attribute another one."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return a[0] if len(a) == 1 and callable(a[0]) and not k else _Anything()

    def __getattr__(self, name):
        return _Anything()

    def __mro_entries__(self, bases):
        return (object,)


def _stub(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    m.__getattr__ = lambda attr: (Exception if attr[:1].isupper() and attr.endswith(("Error", "Converged"))
                                  else type(attr, (), {}))
    m.__path__ = []  # a package: submodules are stubbed on demand below
    sys.modules[name] = m
    return m


class _MultiIndex:
    @staticmethod
    def from_tuples(tuples):
        return [tuple(t) for t in tuples]


def install():
    """Stand-ins for numba, pandas, pandapower; the reference checkout importable as p3s."""
    ref_root = os.path.dirname(os.path.dirname(ob.REF_CPP))
    if not os.path.isdir(os.path.join(ref_root, "p3s")):
        raise RuntimeError(f"reference checkout not found at {ref_root} (set P3S_REFERENCE)")
    if ref_root not in sys.path:
        sys.path.append(ref_root)
    nb = _stub("numba", njit=lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f)), prange=range,
               set_num_threads=lambda n: None, get_num_threads=lambda: 1,
               config=types.SimpleNamespace(NUMBA_NUM_THREADS=1))
    nb.typed = _stub("numba.typed", List=list)
    pd = _stub("pandas", MultiIndex=_MultiIndex, isna=lambda x: x != x)
    pd.api = _stub("pandas.api")
    pp = _stub("pandapower")
    for sub in ("pandapower.auxiliary", "pandapower.toolbox", "pandapower.topology", "pandapower.networks"):
        setattr(pp, sub.split(".")[1], _stub(sub))
    # p3s.NewtonPowerflowCpp imports the compiled nr_klu module: the reference's own build
    ob.build_reference()
    nk = ob.load_reference("fastmath")
    if nk is not None:
        import p3s

        sys.modules["p3s.nr_klu"] = nk
        p3s.nr_klu = nk
