"""The element sources of the run-time compiled assembly compile for sm_103a
(NVRTC runs without a GPU), and a source that does not compile is reported
with the compiler's log."""
import pytest
import torch

from simit_gb300 import _lib, jit_elements
from simit_gb300.runtime import check_element_source


def _check(*a, **k):
    try:
        return check_element_source(*a, **k)
    except _lib.SimitError as e:
        if e.code == _lib.ERR_UNSUPPORTED:
            pytest.skip("NVRTC not available: %s" % e)
        raise


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("name,src,card,bs", [
    ("blocks", jit_elements.BLOCKS, 4, 3),
    ("blocks-wide", jit_elements.BLOCKS, 8, 5),
    ("blocks-edge", jit_elements.BLOCKS, 2, 1),
    ("heat", jit_elements.heat(0.01), 4, 1),
    ("linear-tet", jit_elements.linear_tet(1.0, 1e3), 4, 3),
])
def test_element_sources_compile(name, src, card, bs, dtype):
    _check(src, card, bs, dtype=dtype, exact=True)
    _check(src, card, bs, dtype=dtype, exact=False)


def test_compile_error_carries_the_log():
    with pytest.raises(_lib.SimitError) as ei:
        _check("__device__ int element_block(long long e, int i, int j, const int *ep,\n"
               "  const real *const *f, sg_block *blk) { return undefined_name; }", 2, 1)
    assert ei.value.code == _lib.ERR_ARG
    assert "does not compile" in str(ei.value) and "undefined_name" in str(ei.value)


def test_bad_shape_rejected():
    for card, bs in ((0, 1), (33, 1), (2, 0), (2, 17)):
        with pytest.raises(_lib.SimitError):
            check_element_source(jit_elements.BLOCKS, card, bs)


def test_concurrent_compiles():
    """Several threads compiling at once (the first use loads NVRTC) each get
    their own result and their own error message."""
    from concurrent.futures import ThreadPoolExecutor
    _check(jit_elements.BLOCKS, 2, 1)  # skips when NVRTC is absent

    def one(k):
        if k % 3 == 2:
            try:
                check_element_source("__device__ int element_block(broken %d" % k, 2, 1)
            except _lib.SimitError as e:
                return ("err", str(e))
            return ("ok", "")
        check_element_source(jit_elements.heat(0.01 * (k + 1)), 4, 1,
                             dtype=torch.float32 if k % 2 else torch.float64)
        return ("ok", "")

    with ThreadPoolExecutor(6) as ex:
        res = list(ex.map(one, range(12)))
    for k, (kind, msg) in enumerate(res):
        assert kind == ("err" if k % 3 == 2 else "ok"), (k, msg)
        if kind == "err":
            assert "does not compile" in msg
