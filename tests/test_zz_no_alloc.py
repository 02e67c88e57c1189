"""plk_sum_sites_noalloc: the entry point for callers that cannot allocate
device memory (stream capture, a foreign allocator owning device memory, no
room for cudaMalloc's device synchronisation).  It must give the total that
the ordinary entry point (plk_loglik) gives from the same per-site values,
call after call, although every call reuses one file-scope device array.

Named to be collected last.  Device memory for the test's own inputs comes
from torch; the entry point itself allocates nothing."""
import math

import numpy as np
import pytest

from phylommand_gb300 import plk
import helpers as H

pytestmark = pytest.mark.gpu

REL = 1e-12  # the FP64 tolerance of the parity tests


def test_noalloc_sum_matches_plk_loglik_on_consecutive_calls():
    import torch
    fx = H.load_fixture("syn_gtr_gamma_ambig")
    with H.engine_for_fixture(fx, p_mode=plk.PLK_P_EXACT) as h:
        lnl64 = h.loglik(plk.PLK_FP64)
        site64 = h.site_loglik()
        lnl32 = h.loglik(plk.PLK_FP32S)
        site32 = h.site_loglik()
    dev = torch.device("cuda", 0)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for site, ref in ((site64, lnl64), (site32, lnl32), (site64, lnl64)):
        d = torch.tensor(site, dtype=torch.float64, device=dev)
        out.fill_(float("nan"))
        plk.sum_sites_noalloc(d.data_ptr(), d.numel(), out.data_ptr(), stream)
        torch.cuda.synchronize(dev)
        assert out.item() == pytest.approx(ref, rel=REL)


def test_noalloc_sum_at_the_size_limit_then_smaller():
    """A full-size call followed by a smaller one: the second must not see the
    first call's partial sums left in the shared array."""
    import torch
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(7)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for n in (1_048_576, 1000, 1):
        x = -rng.exponential(3.0, size=n)
        d = torch.tensor(x, dtype=torch.float64, device=dev)
        plk.sum_sites_noalloc(d.data_ptr(), n, out.data_ptr(), stream)
        torch.cuda.synchronize(dev)
        ref = math.fsum(x.tolist())
        assert out.item() == pytest.approx(ref, rel=REL)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    import torch
    dev = torch.device("cuda", 0)
    d = torch.zeros(4, dtype=torch.float64, device=dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    for bad in (0, 1_048_577):
        with pytest.raises(plk.PlkError) as e:
            plk.sum_sites_noalloc(d.data_ptr(), bad, out.data_ptr(), None)
        assert e.value.status == plk.PLK_ERR_ARG
        assert "n_sites" in e.value.message
