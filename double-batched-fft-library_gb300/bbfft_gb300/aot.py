"""Ahead-of-time kernel generation, the counterpart of the reference's bbfft-aot-generate
(tools/aot/main.cpp:22-60, docs/manual/caching.rst: "offline" kernels registered with an
aot_cache at run time).

    python -m bbfft_gb300.aot -o kernels.cubin --callbacks user.cu [--load NAME] [--store NAME]
                              [--arch sm_103a] DESCRIPTOR...

compiles the kernels that the configurations DESCRIPTOR... (reference descriptor
strings, e.g. ``scfo64*1000``) need with the user module of ``--callbacks`` into one cubin
``kernels.cubin`` and writes their names to ``kernels.cubin.names``.  ``--arch`` compiles
for that architecture without a GPU (BBFFT_GB300_AOT_ARCH).  Kernels of configurations
without callbacks are compiled into the library and need no image.  At run time
``load(path)`` returns an aot_cache serving the image; plans made with it need no NVRTC.
"""
import argparse
import os
import sys

import bbfft_gb300 as bb


def generate(descriptors, source, load=None, store=None, arch=None):
    """(image bytes, kernel names) for the descriptors with the given user module."""
    if arch:
        os.environ['BBFFT_GB300_AOT_ARCH'] = arch
    cfgs = []
    for d in descriptors:
        c = bb.parse_fft_descriptor(d)
        cfgs.append(bb.configuration(c.dim, list(c.shape)[:c.dim + 2], precision=c.precision,
                                     direction=c.direction, type=c.type,
                                     istride=list(c.istride), ostride=list(c.ostride),
                                     callbacks=(source, load, store)))
    return bb.aot_generate(cfgs)


def write(path, image, names):
    with open(path, 'wb') as f:
        f.write(image)
    with open(path + '.names', 'w') as f:
        f.write('\n'.join(names) + '\n')


def load(path, device=0):
    """An aot_cache (bbfft_gb300.Cache(aot=True)) serving the image written by write()."""
    with open(path, 'rb') as f:
        image = f.read()
    with open(path + '.names') as f:
        names = [n.strip() for n in f if n.strip()]
    cache = bb.Cache(aot=True)
    cache.register_module(image, names, device)
    return cache


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split('\n\n')[0])
    ap.add_argument('-o', dest='out', required=True, help='output cubin; names go to OUT.names')
    ap.add_argument('--callbacks', required=True, help='CUDA C++ file with the load/store functions')
    ap.add_argument('--load', default=None, help='name of the load callback')
    ap.add_argument('--store', default=None, help='name of the store callback')
    ap.add_argument('--arch', default=None, help='target architecture, e.g. sm_103a (no GPU needed)')
    ap.add_argument('descriptors', nargs='+', help='FFT descriptors, e.g. scfo64*1000')
    a = ap.parse_args(argv)
    if not a.load and not a.store:
        ap.error('name at least one of --load / --store')
    with open(a.callbacks) as f:
        source = f.read()
    image, names = generate(a.descriptors, source, a.load, a.store, a.arch)
    write(a.out, image, names)
    print('wrote %s (%d bytes, %d kernels)' % (a.out, len(image), len(names)))


if __name__ == '__main__':
    sys.exit(main())
