#!/usr/bin/env python3
"""Build the sm_103a library in-tree: bbfft_gb300/_lib/libbbfft_gb300.so.

Translation units are compiled in parallel (nvcc for the kernels, the host compiler
for the host library) and linked with nvcc.  The device engine is also embedded as
text (engine_src.inc) so that plans with user callbacks can be compiled by NVRTC at
run time.  Outputs are rebuilt only when a source is newer than the library.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, 'include')
OUTDIR = os.path.join(HERE, 'bbfft_gb300', '_lib')
# object files and generated sources: outside the source tree (hundreds of MB that a copy of
# the tree should not carry), one directory per checkout; BBFFT_GB300_BUILD_DIR overrides
BUILD = os.environ.get('BBFFT_GB300_BUILD_DIR') or os.path.join(
    tempfile.gettempdir(), 'bbfft_gb300_build_' + hashlib.sha1(HERE.encode()).hexdigest()[:10])
LIB = os.path.join(OUTDIR, 'libbbfft_gb300.so')
# throughput probes for the benchmark's roofline denominators (not part of the library)
PROBES_SRC = os.path.join(CSRC, 'peak_probes.cu')
PROBES_LIB = os.path.join(OUTDIR, 'libbbfft_probes.so')

ARCH = '-gencode=arch=compute_103a,code=sm_103a'
ENGINE_HEADERS = ['params.h', 'root_of_unity_table.cuh', 'radix.cuh', 'engine.cuh']
KERNEL_UNITS = ['kernels_f32.cu', 'kernels_f64.cu', 'noalloc.cu', 'tc.cu', 'strided_copy.cu',
                'bluestein.cu']
# relocatable device code, linked with nvcc -dlink: the persistent ragged kernel calls the
# compile-time-size tile functions of the generated ragged_ct_<i>.cu units
RDC_UNITS = ['ragged.cu']
HOST_UNITS = ['library.cpp', 'config.cpp']


def cuda_home():
    for c in (os.environ.get('CUDA_HOME'), os.environ.get('CUDA_PATH'), '/usr/local/cuda'):
        if c and os.path.exists(os.path.join(c, 'bin', 'nvcc')):
            return c
    nvcc = shutil.which('nvcc')
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError('CUDA toolkit (nvcc) not found')


def embed_engine():
    """Write engine_src.inc: the device engine headers as one raw string for NVRTC."""
    parts = []
    for h in ENGINE_HEADERS:
        with open(os.path.join(CSRC, h)) as f:
            for line in f:
                s = line.strip()
                if s.startswith('#include "') or s == '#pragma once':
                    continue
                parts.append(line)
    text = ''.join(parts)
    out = os.path.join(BUILD, 'engine_src.inc')
    content = ('// generated by build.py from %s\n' % ', '.join(ENGINE_HEADERS) +
               'static const char *kEngineSource = R"GBFFTSRC(\n' + text + '\n)GBFFTSRC";\n')
    if not os.path.exists(out) or open(out).read() != content:
        with open(out, 'w') as f:
            f.write(content)
    return out


def run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError('command failed: %s\n%s' % (' '.join(cmd), r.stdout))
    return r.stdout


def newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def generate_specializations():
    sys.path.insert(0, CSRC)
    import gen_prime_frags
    import gen_specializations

    frag = gen_prime_frags.main(os.path.join(BUILD, 'gen'))
    return gen_specializations.main(os.path.join(BUILD, 'gen')) + (frag,)


def build(verbose=False, jobs=None):
    os.makedirs(OUTDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    cuda = cuda_home()
    nvcc = os.path.join(cuda, 'bin', 'nvcc')
    embed_engine()
    gen_units, rag_units, frag_header = generate_specializations()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC)
               if h.endswith(('.h', '.hpp', '.cuh'))] + [os.path.join(INCLUDE, 'bbfft_gb300.h'),
                                                        frag_header]
    common_inc = ['-I' + CSRC, '-I' + INCLUDE, '-I' + BUILD, '-I' + os.path.join(BUILD, 'gen'),
                  '-I' + os.path.join(cuda, 'include')]
    jobs_list = []
    objs = []
    rdc_objs = []
    for src in [os.path.join(CSRC, u) for u in RDC_UNITS] + rag_units:
        u = os.path.basename(src)
        obj = os.path.join(BUILD, u + '.o')
        rdc_objs.append(obj)
        deps = [src] + headers + [os.path.join(BUILD, 'gen', 'ragged_ct_dispatch.inc')]
        if newer(obj, deps):
            jobs_list.append([nvcc, ARCH, '-lineinfo', '-O3', '-std=c++17', '-rdc=true',
                              '-maxrregcount=128', '-Xcompiler', '-fPIC', '-Xcompiler',
                              '-fvisibility=hidden', '-Xptxas', '-v', '-c', src, '-o', obj] + common_inc)
    for src in [os.path.join(CSRC, u) for u in KERNEL_UNITS] + gen_units:
        u = os.path.basename(src)
        obj = os.path.join(BUILD, u + '.o')
        objs.append(obj)
        if newer(obj, [src] + headers):
            jobs_list.append([nvcc, ARCH, '-lineinfo', '-O3', '-std=c++17', '-Xcompiler', '-fPIC',
                              '-Xcompiler', '-fvisibility=hidden', '-Xptxas', '-v', '-c', src,
                              '-o', obj] + common_inc)
    cxx = os.environ.get('CXX', 'g++')
    for src in [os.path.join(CSRC, u) for u in HOST_UNITS] + [os.path.join(BUILD, 'gen', 'ct_index.cpp')]:
        u = os.path.basename(src)
        obj = os.path.join(BUILD, u + '.o')
        objs.append(obj)
        if newer(obj, [src] + headers + [os.path.join(BUILD, 'engine_src.inc')]):
            jobs_list.append([cxx, '-O2', '-std=c++17', '-fPIC', '-fvisibility=hidden', '-Wall',
                              '-c', src, '-o', obj] + common_inc)
    if newer(PROBES_LIB, [PROBES_SRC]):
        jobs_list.append([nvcc, ARCH, '-lineinfo', '-O3', '-std=c++17', '-shared', '-Xcompiler',
                          '-fPIC', PROBES_SRC, '-o', PROBES_LIB, '-L' + os.path.join(cuda, 'lib64'),
                          '-lcudart'])
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or max(1, os.cpu_count() or 1)) as ex:
            outs = list(ex.map(run, jobs_list))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    dlink = os.path.join(BUILD, 'ragged_dlink.o')
    if newer(dlink, rdc_objs):
        run([nvcc, ARCH, '-dlink', '-Xcompiler', '-fPIC', '-o', dlink] + rdc_objs)
    objs += rdc_objs + [dlink]
    if newer(LIB, objs):
        run([nvcc, ARCH, '-shared', '-Xcompiler', '-fPIC', '-o', LIB] + objs +
            ['-L' + os.path.join(cuda, 'lib64'), '-lcudart', '-lnvrtc'])
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
