"""Build libmcwalk.so (CUDA sm_103a + host C++) in-tree with nvcc and g++.

    python -m monte_carlompi_gb300.build [--force] [--verbose]

Objects go to ``monte_carlompi_gb300/_build/``, the library to
``monte_carlompi_gb300/_lib/libmcwalk.so``.  Translation units compile in
parallel; a unit is rebuilt when any source or header is newer than its object.
"""
import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
VARIANT = os.path.join(BUILD, 'defines_' + ''.join(
    c if c.isalnum() else '_' for c in os.environ['MCW_DEFINES'])) if os.environ.get('MCW_DEFINES') else BUILD
LIBDIR = os.path.join(PKG, '_lib')
LIB = os.path.join(LIBDIR, 'libmcwalk.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']

# units whose FP64 arithmetic must keep the reference's rounding: no contraction
NO_FMAD = {'walk_replay.cu', 'ssp_lut.cu'}
# the FP32 production walk: flush denormals, approximate division and square root
FAST_F32 = {'walk_f32.cu': ['-ftz=true', '-prec-div=false', '-prec-sqrt=false']}
# tuning builds: extra -D flags for the FP32 walk and the fused inference kernel
# (e.g. MCW_DEFINES="-DMCW_BLOCK_WALK=128");
# its object goes to a directory of its own, the other units are shared with the default build
DEFINES = os.environ.get('MCW_DEFINES', '').split()
DEFINE_UNITS = {'walk_f32.cu', 'mlp_fused.cu'}


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _headers():
    return glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(ROOT, 'include', '*.h'))


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


def _compile(src, verbose):
    name = os.path.basename(src)
    obj = os.path.join(VARIANT if name in DEFINE_UNITS else BUILD, name + '.o')
    if not _stale(obj, src):
        return obj, None
    if name.endswith('.cu'):
        defs = DEFINES if name in DEFINE_UNITS else []
        cmd = [nvcc(), *ARCH, '-O3', '-lineinfo', '-std=c++17', *defs, '-Xcompiler', '-fPIC', '-c', src, '-o', obj]
        if name in NO_FMAD:
            cmd.insert(-4, '--fmad=false')
        for flag in FAST_F32.get(name, []):
            cmd.insert(-4, flag)
        if verbose:
            cmd.insert(-4, '-Xptxas=-v')
    else:
        cmd = [os.environ.get('CXX', 'g++'), '-O2', '-std=c++17', '-fPIC', '-Wall', '-c', src, '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('compile failed: %s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))
    return obj, (r.stdout + r.stderr) if verbose else None


def build(force=False, verbose=False):
    """Compile every unit under csrc/ and link libmcwalk.so.  Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(VARIANT, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')) + glob.glob(os.path.join(CSRC, '*.cpp')))
    if force:
        for s in srcs:
            o = os.path.join(VARIANT if os.path.basename(s) in DEFINE_UNITS else BUILD,
                             os.path.basename(s) + '.o')
            if os.path.exists(o):
                os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log, file=sys.stderr)
    stamp = LIB + '.objdir'     # which object directory the library was linked from
    same_dir = os.path.exists(stamp) and open(stamp).read() == VARIANT
    if force or not same_dir or not os.path.exists(LIB) or \
            any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, '-shared', '-o', LIB, *objs, '-lpthread']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed: %s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))
        with open(stamp, 'w') as f:
            f.write(VARIANT)
    return LIB


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--force', action='store_true')
    ap.add_argument('--verbose', action='store_true')
    a = ap.parse_args()
    print(build(a.force, a.verbose))
