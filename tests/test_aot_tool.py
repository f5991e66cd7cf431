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


ND_SRC = """
float2 load_id(float2 *in, size_t offset) { return in[offset]; }
void store_id(float2 *out, size_t offset, float2 v) { out[offset] = v; }
void store_id(float *out, size_t offset, float v) { out[offset] = v; }
"""


def test_aot_tool_nd_configurations(bb, tmp_path):
    """nd configurations with callbacks need two kernels each: the first pass calls the load
    function, the last pass the store function (c2r: the c2c pass first, its real pass last);
    a 1d configuration needs one kernel calling both."""
    from bbfft_gb300 import aot

    src = tmp_path / 'user.cu'
    src.write_text(ND_SRC)
    out = tmp_path / 'nd.cubin'
    old = os.environ.get('BBFFT_GB300_AOT_ARCH')
    try:
        aot.main(['-o', str(out), '--callbacks', str(src), '--load', 'load_id', '--store', 'store_id',
                  '--arch', 'sm_103a', 'scfo8x8*4', 'scbo8x8*4', 'srbo16x8*4', 'scfo64*16'])
    finally:
        if old is None:
            os.environ.pop('BBFFT_GB300_AOT_ARCH', None)
        else:
            os.environ['BBFFT_GB300_AOT_ARCH'] = old
    names = (tmp_path / 'nd.cubin.names').read_text().split()
    assert out.read_bytes()[:4] == b'\x7fELF'
    assert len(names) == len(set(names)) == 4, names
    # the 1d configuration calls both functions in its one pass
    assert sum(n.startswith('gbfft_cb_f32_c2c_load_id_store_id_') for n in names) == 1, names
    assert sum(n.startswith('gbfft_cb_f32_c2c_load_id__') for n in names) == 1, names
    assert sum(n.startswith('gbfft_cb_f32_c2c__store_id_') for n in names) == 1, names
    assert sum(n.startswith('gbfft_cb_f32_c2rh__store_id_') for n in names) == 1, names
