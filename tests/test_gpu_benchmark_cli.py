"""The reference-style benchmark CLI on the GPU: every row is checked against an FP64 DFT
inside the tool (it exits on a mismatch) and reports positive bandwidth."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('argv', [['-o', '-m', '8', '-b', '64m', 'sr', '64', '160'],
                                  ['-i', '-v', '-m', '4', '-b', '32m', 'sr', '96'],
                                  ['-o', '-b', '32m', 'sc', '64', '120'],
                                  ['-i', '-v', '-k', '100', 'dc', '48'],
                                  ['-o', '-m', '2', '-k', '300', 'dr', '13']])
def test_cli_rows(bb, torch_cuda, capsys, argv):
    from bbfft_gb300 import benchmark as bm

    bm.main(argv)
    lines = capsys.readouterr().out.strip().splitlines()
    cols = lines[0].split(',')
    assert cols[:10] == ['p', 'N', 'inplace', 'M', 'K', 'domain', 'inverse', 'time', 'bw', 'flops']
    for line in lines[1:]:
        row = dict(zip(cols, line.split(',')))
        assert float(row['bw']) > 0 and float(row['rel_l2']) < 2e-6
