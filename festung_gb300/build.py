"""Builds ``festung_gb300/libdgadv.so`` in-tree (host C++ + CUDA for sm_103a).

Usage: ``python -m festung_gb300.build`` (or ``festung_gb300.build.build()``).  The translation
units (host helpers, C-ABI, one unit of kernels per arithmetic type, the no-allocation limiter)
compile in parallel; the result is git-ignored.  Host code uses
``-ffp-contract=off`` so that grid and table arithmetic rounds as written on x86-64 and aarch64.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT = os.path.join(HERE, 'libdgadv.so')
BUILD = os.path.join(HERE, '_build')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _cuda_home():
    for c in (os.environ.get('CUDA_HOME'), '/usr/local/cuda'):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which('nvcc')
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError('CUDA toolkit not found (set CUDA_HOME)')


def sources():
    return [os.path.join(CSRC, f) for f in ('dgadv_host.cpp', 'dgadv_capi.cpp', 'dgadv_solver.cu',
                                            'dgadv_prec_fp64.cu', 'dgadv_prec_fp32.cu',
                                            'dgadv_prec_df32_p01.cu', 'dgadv_prec_df32_p2.cu',
                                            'dgadv_prec_df32_p3.cu', 'dgadv_adjoint.cu',
                                            'dgadv_noalloc.cu', 'dgadv_vis.cpp', 'dgadv_output.cu',
                                            'dgadv_setup.cu', 'dgadv_implicit.cu', 'dgadv_transport.cu')]


# per-unit extra flags: the set-up unit evaluates quadrature points and indicator functions
# with separate roundings, as the host expressions do
EXTRA_FLAGS = {'dgadv_setup.cu': ['-fmad=false']}


def _stale():
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, '..', 'include', 'dgadv.h'))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, extra_nvcc=()):
    if not force and not _stale():
        return OUT
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, 'bin', 'nvcc')
    os.makedirs(BUILD, exist_ok=True)
    inc = ['-I', os.path.join(HERE, '..', 'include'), '-I', CSRC]
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src) + '.o')
        objs.append(obj)
        if src.endswith('.cu'):
            cmd = [nvcc, '-O3', '-std=c++17', *ARCH, '-lineinfo', '-Xcompiler', '-fPIC,-ffp-contract=off',
                   *inc, *extra_nvcc, *EXTRA_FLAGS.get(os.path.basename(src), []), '-c', src, '-o', obj]
        else:
            cmd = ['g++', '-O2', '-std=c++17', '-fPIC', '-pthread', '-ffp-contract=off', *inc, '-I',
                   os.path.join(cuda, 'include'), '-c', src, '-o', obj]
        jobs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, pr in jobs:
        out, _ = pr.communicate()
        if verbose or pr.returncode:
            sys.stderr.write(out.decode(errors='replace'))
        if pr.returncode:
            failed.append(' '.join(cmd))
    if failed:
        raise RuntimeError('build failed:\n' + '\n'.join(failed))
    tmp = OUT + '.tmp'
    link = [nvcc, '-shared', *ARCH, '-o', tmp, *objs, '-lcudart', '-Xcompiler', '-pthread']
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode:
        raise RuntimeError('link failed:\n' + r.stdout.decode(errors='replace'))
    os.replace(tmp, OUT)
    return OUT


if __name__ == '__main__':
    build(force='--force' in sys.argv, verbose=True)
    print(OUT)
