"""The C++ API (include/bbfft/*.hpp, header-only over the C ABI), compiled with g++ and
linked against the in-tree library, used the way the reference's callers use theirs."""
import os
import subprocess

import pytest

from conftest import PKG, REPO


@pytest.fixture(scope='module')
def api_test_binary(bb, tmp_path_factory):
    import build as pkg_build

    cuda = pkg_build.cuda_home()
    out = str(tmp_path_factory.mktemp('cpp') / 'api_test')
    libdir = os.path.join(PKG, 'bbfft_gb300', '_lib')
    cmd = ['g++', '-std=c++17', '-O1', '-Wall', '-I', os.path.join(REPO, 'include'),
           '-I', os.path.join(cuda, 'include'), os.path.join(REPO, 'tests', 'cpp', 'api_test.cpp'),
           '-o', out, '-L', libdir, '-lbbfft_gb300', '-Wl,-rpath,' + libdir,
           '-L', os.path.join(cuda, 'lib64'), '-lcudart', '-Wl,-rpath,' + os.path.join(cuda, 'lib64')]
    subprocess.run(cmd, check=True)
    return out


def test_cpp_api_host(api_test_binary):
    r = subprocess.run([api_test_binary, 'host'], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert 'host ok' in r.stdout


@pytest.mark.gpu
def test_cpp_api_gpu(api_test_binary, torch_cuda):
    r = subprocess.run([api_test_binary, 'gpu'], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert 'gpu ok' in r.stdout
