"""The bounded-wait failure path of the tensor-core walk, made to run out.

Every mbarrier wait of the A = 64 tensor-core walk is bounded; a wait that
gives up records the failure in the plan's device status word, which
subby_plan_status (device-pointer runs) or the call itself (host-pointer
runs) reports as SUBBY_ERR_TIMEOUT.  The test hook subby_debug_fail_waits
makes the walk's prologue wait on an mbarrier that nothing arms, while no
copy or MMA is in flight, for a few polls: the wait gives up, the CTA frees
its tensor memory and returns.  The host must then see SUBBY_ERR_TIMEOUT,
and the context must stay usable: the next run, with the hook off, matches
the oracle.  Nothing here faults or hangs the GPU: the wait is bounded and
its failure is the designed outcome.
"""
import numpy as np
import pytest

import oracle
from tests._tol import assert_cols, assert_loglike, COUNTS_RTOL

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import _lib, synth, models  # noqa: E402


def test_walk_wait_gives_up_and_host_sees_timeout():
    rng = np.random.default_rng(91)
    model, _, _ = models.random_reversible(64, rng, 0.5, 2.0)
    tree = synth.random_tree(9, 0.1, rng)
    aln = synth.simulated_alignment(tree, model, 300, 0.1, rng)
    plan = sg.Plan(tree, model)
    d_aln = torch.as_tensor(aln).cuda()
    lib = _lib.load()
    assert lib.subby_debug_fail_waits(-1) == _lib.ERR_ARG
    try:
        assert lib.subby_debug_fail_waits(8) == 0
        # device pointers: the run only enqueues; the status check reports it
        plan.run(d_aln, loglike=True, counts=True, branch_mask=None)
        with pytest.raises(_lib.SubbyError) as e:
            plan.status()
        assert e.value.code == _lib.ERR_TIMEOUT
        assert "gave up" in str(e.value)
        # the record is cleared by the check
        plan.status()
        # host pointers: the call itself reports it
        with pytest.raises(_lib.SubbyError) as e:
            plan.run(aln, loglike=True, counts=True, branch_mask=None)
        assert e.value.code == _lib.ERR_TIMEOUT
    finally:
        lib.subby_debug_fail_waits(0)
    torch.cuda.synchronize()
    # the context is usable and results are right again
    r = plan.run(d_aln, loglike=True, counts=True, branch_mask=None)
    plan.status()
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    md = model._asdict()
    assert_loglike(r['logLike'].cpu().numpy(), oracle.LogLike(aln, ot, md))
    assert_cols(r['counts'].cpu().numpy(), oracle.Counts(aln, ot, md, branch_mask=None), COUNTS_RTOL, "counts")
    plan.close()
