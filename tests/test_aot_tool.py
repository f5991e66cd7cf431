"""The ahead-of-time tool (bbfft_gb300.aot, the bbfft-aot-generate counterpart): compiles
callback kernels for an architecture named on the command line, without a GPU."""
import os


SRC = "float2 load_id(float2 *in, size_t offset) { return in[offset]; }\n"


def test_aot_tool_offline(bb, tmp_path):
    from bbfft_gb300 import aot

    src = tmp_path / 'user.cu'
    src.write_text(SRC)
    out = tmp_path / 'kernels.cubin'
    old = os.environ.get('BBFFT_GB300_AOT_ARCH')
    try:
        aot.main(['-o', str(out), '--callbacks', str(src), '--load', 'load_id', '--arch', 'sm_103a',
                  'scfo64*16', 'scbo64*16', 'scfo128*8'])
    finally:
        if old is None:
            os.environ.pop('BBFFT_GB300_AOT_ARCH', None)
        else:
            os.environ['BBFFT_GB300_AOT_ARCH'] = old
    image = out.read_bytes()
    names = (tmp_path / 'kernels.cubin.names').read_text().split()
    assert image[:4] == b'\x7fELF' and len(image) > 1000
    # c2c forward and backward share one kernel kind; every name is unique
    assert len(names) == len(set(names)) >= 1
