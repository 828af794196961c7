"""The package entry's smoke(): one small S(Q,omega) job on cuda:0 through the C ABI, checked
against the oracle; it raises on any mismatch."""
import pytest


@pytest.mark.gpu
def test_entry_smoke(cuda):
    import __graft_entry__
    __graft_entry__.smoke()
