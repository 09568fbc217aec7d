"""Two frames in flight (sw_set_frames_in_flight): a call returns once its frame is enqueued and the
previous frame is in its host buffer, the copy into host memory overlapping the next frame's work. The
frames and the exposure sequence must equal those of one frame at a time, for both preparation splits."""
import ctypes

import numpy as np
import pytest

from sqwheel import abi, gpu, host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("gpu_prep", [True, False])
def test_frames_in_flight_equal_serial(gpu_ok, gpu_prep):
    scene = host.Scene(**dict(host.FULL_MAP, grid_x=4, grid_y=4))
    opts = host.frame_options(640, 360, abi.SW_PIXEL_C64, directional=True)
    cfg = abi.PostConfig.default()
    frames = [0, 9, 17, 18, 40, 77, 78, 120]
    glib = gpu.load_library()
    serial = host.HostRenderer(scene)
    serial.set_gpu_prep(gpu_prep)
    piped = host.HostRenderer(scene)
    piped.set_gpu_prep(gpu_prep)
    piped.set_frames_in_flight(2)
    bufs = [np.zeros((360, 640), np.uint32), np.zeros((360, 640), np.uint32)]
    want, want_exposure = [], []
    e = ctypes.c_float()
    try:
        out = np.zeros((360, 640), np.uint32)
        for fi in frames:
            serial.render_frame(fi, opts, out=out, post=cfg)
            want.append(out.copy())
            glib.sw_get_exposure(serial.context(), ctypes.byref(e))
            want_exposure.append(e.value)
        for b in bufs:
            piped.register_host_buffer(b)
        for k, fi in enumerate(frames):
            piped.render_frame(fi, opts, out=bufs[k % 2], post=cfg)
            if k > 0:  # the previous frame is in its buffer when the call returns
                assert np.array_equal(bufs[(k - 1) % 2], want[k - 1]), f"frame {frames[k - 1]} differs"
        piped.sync()
        assert np.array_equal(bufs[(len(frames) - 1) % 2], want[-1])
        glib.sw_get_exposure(piped.context(), ctypes.byref(e))
        assert e.value == np.float32(want_exposure[-1])
        for b in bufs:
            piped.unregister_host_buffer(b)
    finally:
        serial.close()
        piped.close()
