"""The C-ABI library loads and exports every symbol include/m3sph.h declares (no GPU calls)."""
import re
from pathlib import Path

import ctypes

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    h = (ROOT / 'include' / 'm3sph.h').read_text()
    return sorted(set(re.findall(r'M3SPH_API\s+[^;]*?\b(m3sph_\w+)\s*\(', h)))


def test_library_exports_header_symbols(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    from m3tet_sph_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_no_cpu_fallback_in_product(built_lib):
    """The package never imports the oracle."""
    for p in (ROOT / 'm3tet_sph_gb300').rglob('*.py'):
        assert 'oracle' not in re.sub(r'#.*', '', p.read_text()).replace('oracle is', ''), p
