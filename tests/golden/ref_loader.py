"""Load the reference's ``pyqed.oqs`` without its package ``__init__``.

Used only by ``make_golden.py`` in a container where the reference sources are
mounted (read-only); the environment variable ``PYQED_REFERENCE`` names the
directory that holds the reference's ``pyqed`` package.  ``import pyqed`` fails there
(missing matplotlib/gbasis and a circular import in ``pyqed/__init__.py:9``
-> ``pyqed/qchem``), so this registers an empty ``pyqed`` package whose
``__path__`` is the reference tree, stubs the plotting packages that
``pyqed/signal/sos.py`` and ``pyqed/style.py`` import at module level, then
imports ``pyqed.phys``, ``pyqed.units``, ``pyqed.mol`` and ``pyqed.oqs``.
"""
import os, sys, types, importlib, importlib.abc, importlib.machinery
_STUB_ROOTS = ('matplotlib', 'proplot', 'mpl_toolkits')

class _Stub(types.ModuleType):
    def __getattr__(self, k):
        if k.startswith('__'):
            raise AttributeError(k)
        return _Stub(self.__name__ + '.' + k)
    def __call__(self, *a, **kw):
        return _Stub(self.__name__ + '()')

class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, name, path, target=None):
        if name.split('.')[0] in _STUB_ROOTS:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None
    def create_module(self, spec):
        m = _Stub(spec.name); m.__path__ = []
        return m
    def exec_module(self, module):
        pass

def load():
    if 'pyqed.oqs' in sys.modules:
        return sys.modules['pyqed.oqs']
    ref = os.environ.get('PYQED_REFERENCE')
    if not ref or not os.path.isdir(os.path.join(ref, 'pyqed')):
        raise RuntimeError('set PYQED_REFERENCE to the directory holding the reference pyqed package')
    sys.meta_path.insert(0, _StubFinder())
    pkg = types.ModuleType('pyqed'); pkg.__path__ = [os.path.join(ref, 'pyqed')]
    sys.modules['pyqed'] = pkg
    phys = importlib.import_module('pyqed.phys')
    units = importlib.import_module('pyqed.units')
    for mod in (phys, units):
        for k in dir(mod):
            if not k.startswith('_'):
                setattr(pkg, k, getattr(mod, k))
    mol = importlib.import_module('pyqed.mol')
    pkg.Mol = mol.Mol; pkg.Result = mol.Result
    oqs = importlib.import_module('pyqed.oqs')
    return oqs
