"""The BLContext binding's function table, without a device: every BLContextVirt slot is set and
the slots the backend does not support answer BL_ERROR_NOT_IMPLEMENTED (the behaviour a caller of
an unsupported BLContext feature sees)."""
import pytest

import blcontext_lib

pytestmark = pytest.mark.skipif(not blcontext_lib.available(), reason="reference sources not staged (oracle/stage_ref.sh)")


def test_virt_table_is_complete_and_unsupported_slots_say_so():
    rc, out, err = blcontext_lib.run("--virt")
    assert rc == 0, (out, err)
    assert out["null_slots"] == 0 and out["slots"] >= 80
