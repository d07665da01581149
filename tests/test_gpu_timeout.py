"""Failure detection without a GPU fault: every wait inside the frame kernels (the
software grid barrier between the phases of a cooperative launch and the bulk-copy
waits of meshlet tiles) is bounded. A test limit of a few polls makes the waits give
up on a frame that runs many blocks; the kernel records the timeout and every block
leaves, the host reports T3D_E_TIMEOUT with a message, and the context stays usable:
the next frame, with the default limit, is bit-identical to the oracle. Nothing
faults, traps or hangs. The batched frame as one cooperative launch always waits on
its grid barriers. The batched frame as one launch per phase and the plain form have
no grid barrier: without meshlets they have no wait at all and the frame renders; with
meshlets only the bulk-copy waits are bounded, and those may finish within the test
limit, so that frame either gives up or renders, bit-exact either way."""
import pytest

from tetra3d_gb300 import abi, scenes
from oracle import pyoracle
from tests.parity import assert_frames_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("meshlets", [1, 0])
@pytest.mark.parametrize("mode,split", [(abi.MODE_BATCHED, 0), (abi.MODE_BATCHED, 1), (abi.MODE_PLAIN, 1)])
def test_bounded_waits_give_up_and_the_next_frame_renders(ctx, meshlets, mode, split):
    sd = scenes.small_variant("batched", 21)
    ctx.set_meshlets(meshlets)
    ctx.set_split_phases(split)
    sid = ctx.upload(sd)
    try:
        ctx.set_wait_limit(2)
        ctx.render(sid, sd.camera, mode=mode)
        if mode == abi.MODE_PLAIN or split:
            try:
                assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), "plain form, tiny wait limit")
            except abi.T3DError as e:
                assert meshlets and e.code == abi.T3D_E_TIMEOUT, (meshlets, e.code)
                assert "error" in str(e)
        else:
            with pytest.raises(abi.T3DError) as e:
                ctx.sync()
            assert e.value.code == abi.T3D_E_TIMEOUT
            assert "error" in str(e.value)
        ctx.set_wait_limit(0)
        ctx.render(sid, sd.camera, mode=mode)
        assert_frames_equal(ctx.download(), pyoracle.render(sd, sd.camera), f"after timeout, meshlets={meshlets}")
    finally:
        ctx.set_wait_limit(0)
        ctx.set_meshlets(1)
        ctx.set_split_phases(1)
        ctx.release(sid)
