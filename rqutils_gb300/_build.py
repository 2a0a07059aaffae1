"""Compile the CUDA sources of rqutils_gb300 into one shared library (in-tree, sm_103a).

    python -m rqutils_gb300._build          # or __graft_entry__.build()

Every ``csrc/*.cu`` file is compiled to an object in parallel with nvcc, then linked into
``rqutils_gb300/_lib/librqsqd.so`` (static CUDA runtime, only the ``rq_*`` C ABI exported).
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
OUTDIR = os.path.join(HERE, '_lib')
OBJDIR = os.path.join(ROOT, '_build', 'obj')
LIBNAME = 'librqsqd.so'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '--expt-relaxed-constexpr', '-Xcompiler', '-fPIC',
         '-Xcompiler', '-fvisibility=hidden', '-I', INCLUDE, '-I', CSRC]


def nvcc():
    exe = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(exe):
        raise RuntimeError('nvcc not found')
    return exe


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _headers_digest():
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            if f.endswith(('.h', '.cuh')):
                with open(os.path.join(d, f), 'rb') as fh:
                    h.update(fh.read())
    h.update(' '.join(ARCH + FLAGS).encode())
    return h.hexdigest()[:16]


def _compile(src, obj, verbose):
    cmd = [nvcc()] + ARCH + FLAGS + ['-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}')
    return r.stderr if verbose else ''


def build(force=False, verbose=False, jobs=None):
    """Build (or rebuild when sources changed) and return the path of the shared library."""
    os.makedirs(OUTDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    lib = os.path.join(OUTDIR, LIBNAME)
    digest = _headers_digest()
    stamp = os.path.join(OBJDIR, 'headers.stamp')
    stale_headers = force or not os.path.exists(stamp) or open(stamp).read() != digest
    todo = []
    objs = []
    for src in _sources():
        obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + '.o')
        objs.append(obj)
        if stale_headers or not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src):
            todo.append((src, obj))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(todo))) as ex:
            logs = list(ex.map(lambda so: _compile(so[0], so[1], verbose), todo))
        if verbose:
            for log in logs:
                sys.stderr.write(log)
    if todo or not os.path.exists(lib):
        tmp = lib + '.tmp'
        cmd = [nvcc()] + ARCH + ['-shared', '-o', tmp] + objs + ['-Xcompiler', '-fvisibility=hidden']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'link failed:\n{r.stdout}\n{r.stderr}')
        os.replace(tmp, lib)
    with open(stamp, 'w') as fh:
        fh.write(digest)
    return lib


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
