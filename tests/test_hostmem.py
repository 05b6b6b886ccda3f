"""hostmem without a GPU: registration fails cleanly (an error from the
library, nothing left registered or mapped)."""
import pytest

from conftest import pkg

torch = pytest.importorskip("torch")


@pytest.mark.skipif(torch.cuda.is_available(), reason="needs a machine without a CUDA device")
def test_register_failure_is_clean():
    hm = pkg("hostmem")
    with pytest.raises(RuntimeError, match="pjg_host_register"):
        hm.empty((1024,))
    assert not hm._keep


def test_empty_of_size_zero_needs_no_registration():
    hm = pkg("hostmem")
    a = hm.empty((0, 5))
    assert a.shape == (0, 5) and not hm._keep
