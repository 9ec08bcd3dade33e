"""The run-time-specialised kernels' generated source compiles with NVRTC for sm_103a (CPU
test: NVRTC needs no GPU). ``ops`` > 0 selects the fused sweep with that op set, -1 the forward
rollout kernel, -2 / -3 the RNEA / ABA vector-Jacobian product kernels, -4 / -5 / -6 the forward
rollout, the backward's reverse sweep and forward dynamics alone with three lanes per
environment, -7 the CRBA + RNEA + ABA sweep as one warp per role of a team. GPU parity of the specialised kernels is in
test_jit_gpu.py."""
import ctypes
import ctypes.util

import pytest

from sapien_gb300 import PinocchioModel, synthetic as syn
from sapien_gb300 import _native as N


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("libnvrtc not available")


def _headers():
    import os

    from sapien_gb300.build_native import CSRC, JIT_HEADERS

    return [h.encode() for h in JIT_HEADERS], [open(os.path.join(CSRC, h)).read().encode() for h in JIT_HEADERS]


@pytest.mark.parametrize("name,ops", [("arm9", 31), ("arm9", 3), ("humanoid", 28), ("mixed", 8), ("arm9", -1),
                                      ("mixed", -1), ("quadruped", -1), ("arm9", -2), ("humanoid", -3),
                                      ("arm9", -4), ("mixed", -4), ("arm9", -5), ("chain40", -5), ("arm9", -6),
                                      ("humanoid", -7)])
def test_generated_source_compiles(name, ops):
    robot = {"arm9": syn.arm_with_fingers(), "humanoid": syn.humanoid(), "quadruped": syn.quadruped(),
             "chain40": syn.serial_chain(40, seed=23),
             "mixed": syn.serial_chain(6, seed=11, kinds=["revolute", "continuous", "prismatic", "revolute",
                                                          "continuous", "prismatic"])}[name]
    pm = PinocchioModel(robot.urdf, [0, 0, -9.81])
    pm.set_joint_order(robot.joint_names)
    pm.set_link_order(robot.link_names)
    if ops == -7:  # one warp per role of a 4-lane team
        pm.set_lanes(4)
    src = ctypes.c_char_p()
    assert N.load().sgdyn_jit_source(pm._h, ops, ctypes.byref(src)) == 0
    nv = _nvrtc()
    names, texts = _headers()
    prog = ctypes.c_void_p()
    arr = lambda xs: (ctypes.c_char_p * len(xs))(*xs)  # noqa: E731
    assert nv.nvrtcCreateProgram(ctypes.byref(prog), src.value, b"sgjit_kernel.cu", len(names), arr(texts),
                                 arr(names)) == 0
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"-lineinfo"]
    rc = nv.nvrtcCompileProgram(prog, len(opts), arr(opts))
    if rc != 0:
        n = ctypes.c_size_t()
        nv.nvrtcGetProgramLogSize(prog, ctypes.byref(n))
        log = ctypes.create_string_buffer(n.value)
        nv.nvrtcGetProgramLog(prog, log)
        pytest.fail(log.value.decode()[:3000])
    size = ctypes.c_size_t()
    assert nv.nvrtcGetCUBINSize(prog, ctypes.byref(size)) == 0 and size.value > 1000
    nv.nvrtcDestroyProgram(ctypes.byref(prog))
