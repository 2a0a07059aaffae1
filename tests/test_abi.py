"""The C ABI library builds, loads and exports exactly what include/rqsqd.h declares (CPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'rqsqd.h')


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    names = re.findall(r'^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(rq_[a-z0-9_]+)\s*\(', src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope='module')
def libpath():
    from rqutils_gb300._build import build
    return build()


def test_header_parses():
    names = declared_functions()
    assert 'rq_matvec' in names and 'rq_lobpcg_solve' in names and len(names) >= 14


def test_exports_match_header(libpath):
    out = subprocess.run(['nm', '-D', '--defined-only', libpath], capture_output=True, text=True,
                         check=True).stdout
    exported = sorted(set(re.findall(r' T (rq_[a-z0-9_]+)$', out, flags=re.M)))
    assert exported == declared_functions()


def test_ctypes_binding_covers_header(libpath):
    from rqutils_gb300 import _lib as L
    assert sorted(L.SIGNATURES) == declared_functions()
    lib = L.lib()
    assert lib.rq_version() >= 100
    for name in declared_functions():
        assert hasattr(lib, name)


def test_host_only_entry_points(libpath):
    """Sizing calls need no GPU."""
    from rqutils_gb300 import _lib as L
    lib = L.lib()
    hb = ctypes.c_int32()
    assert lib.rq_subspace_sizes(1 << 20, 64, ctypes.byref(hb)) == 0
    assert (4 << hb.value) >= 8 * (1 << 20) and (4 << (hb.value - 1)) < 8 * (1 << 20)
    assert lib.rq_subspace_sizes(1 << 20, 32, ctypes.byref(hb)) == 0
    assert (4 << hb.value) >= 8 * (1 << 20)
    n = ctypes.c_size_t()
    assert lib.rq_scratch_size(1 << 20, ctypes.byref(n)) == 0 and n.value > 0
    pb = ctypes.c_int32()
    assert lib.rq_presence_bits(1 << 20, 32, ctypes.byref(pb)) == 0 and pb.value == 0
    assert lib.rq_presence_bits(1 << 26, 64, ctypes.byref(pb)) == 0 and pb.value == 29
    assert lib.rq_presence_bits(1 << 22, 64, ctypes.byref(pb)) == 0 and pb.value == 25
    prm = L.LobpcgParams(maxiter=10, variant=0, vtype=L.C128, mixed=1)
    assert lib.rq_lobpcg_workspace_size(1000, ctypes.byref(prm), ctypes.byref(n)) == 0
    assert n.value >= 8 * 1000 * 24
    assert lib.rq_subspace_sizes(0, 64, ctypes.byref(hb)) == L.E_ARG
    assert b'D must be' in lib.rq_last_error()
    # line filter: two states per 256-bit line, 2^(lbits + lwbits - 3) bytes; at most 2^(37 -
    # lwbits) lines, so that a word index fits 32 bits
    lb = ctypes.c_int32()
    assert lib.rq_line_filter_bits(1 << 20, 8, ctypes.byref(lb)) == 0 and lb.value == 19
    assert lib.rq_line_filter_bits(1 << 20, 10, ctypes.byref(lb)) == 0 and lb.value == 17
    assert lib.rq_line_filter_bits(3, 8, ctypes.byref(lb)) == 0 and lb.value == 1
    assert lib.rq_line_filter_bits((1 << 31) - 1, 8, ctypes.byref(lb)) == 0 and lb.value == 29
    assert lib.rq_line_filter_bits((1 << 31) - 1, 10, ctypes.byref(lb)) == 0 and lb.value == 27
    assert lib.rq_line_filter_bits(1 << 20, 11, ctypes.byref(lb)) == L.E_ARG


def test_lobpcg_parameters_validated_on_the_host(libpath):
    """rq_lobpcg_solve rejects a negative restart period (and a negative maxiter) before it
    touches the device."""
    from rqutils_gb300 import _lib as L
    lib = L.lib()
    op = L.Operator()
    op.sub.D = 16
    res = L.LobpcgResult()
    dummy = ctypes.c_void_p(16)  # never dereferenced: validation fails first
    prm = L.LobpcgParams(maxiter=10, variant=L.LOBPCG_FAST, vtype=L.C128, restart=-1)
    assert lib.rq_lobpcg_solve(ctypes.byref(op), ctypes.byref(prm), dummy, dummy, dummy,
                               ctypes.byref(res), None) == L.E_ARG
    assert b'restart' in lib.rq_last_error()
    prm = L.LobpcgParams(maxiter=-1, variant=L.LOBPCG_FAST, vtype=L.C128)
    assert lib.rq_lobpcg_solve(ctypes.byref(op), ctypes.byref(prm), dummy, dummy, dummy,
                               ctypes.byref(res), None) == L.E_ARG


def test_struct_layouts():
    from rqutils_gb300 import _lib as L
    assert ctypes.sizeof(L.Subspace) == 112
    assert ctypes.sizeof(L.Terms) == 56
    assert ctypes.sizeof(L.Operator) == 112 + 56 + 8 + 40 + 8
    assert ctypes.sizeof(L.LobpcgParams) == 72
    assert ctypes.sizeof(L.LobpcgResult) == 48
    assert ctypes.sizeof(L.Batch) == 240
    assert L.Batch.terms.offset == 80 and L.Batch.nnz.offset == 184
    assert ctypes.sizeof(L.Mlp) == 56


def test_terms_upload_validates_on_the_host(libpath):
    """rq_terms_upload rejects a bad grouping before it touches the device."""
    import numpy as np
    from rqutils_gb300 import _lib as L
    lib = L.lib()
    t = L.Terms()
    dummy = ctypes.c_void_p(16)  # never dereferenced: validation fails first
    xm = np.array([3, 1], np.uint64)            # not increasing
    toff = np.array([0, 1, 2], np.int32)
    zm = np.zeros(2, np.uint64)
    cf = np.zeros(4, np.float64)
    args = [xm.ctypes.data, toff.ctypes.data, zm.ctypes.data, cf.ctypes.data] + [dummy] * 5
    assert lib.rq_terms_upload(2, 2, *args, ctypes.byref(t), None) == L.E_ARG
    assert b'increasing' in lib.rq_last_error()
    xm2 = np.array([1, 3], np.uint64)
    bad = np.array([0, 2, 1], np.int32)          # does not end at K
    args = [xm2.ctypes.data, bad.ctypes.data, zm.ctypes.data, cf.ctypes.data] + [dummy] * 5
    assert lib.rq_terms_upload(2, 2, *args, ctypes.byref(t), None) == L.E_ARG


def test_struct_layouts_match_the_c_header(tmp_path):
    """The ctypes structures have the sizes and field offsets the C compiler gives the header's
    structures (gcc on include/rqsqd.h)."""
    import shutil
    import subprocess
    from rqutils_gb300 import _lib as L
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    structs = {'rq_subspace_t': L.Subspace, 'rq_terms_t': L.Terms, 'rq_operator_t': L.Operator,
               'rq_lobpcg_params_t': L.LobpcgParams, 'rq_lobpcg_result_t': L.LobpcgResult,
               'rq_batch_t': L.Batch}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rqsqd.h"', 'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'printf("{cname}.{f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ['return 0;', '}']
    src = tmp_path / 'layout.c'
    src.write_text('\n'.join(lines))
    exe = tmp_path / 'layout'
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'include')
    subprocess.run([cc, '-I', inc, str(src), '-o', str(exe)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], check=True, capture_output=True,
                                                    text=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert int(got[f'{cname}.{f[0]}']) == getattr(py, f[0]).offset, (cname, f[0])
