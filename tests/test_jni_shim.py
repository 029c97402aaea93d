"""The JNI binding's native half (dayflower-path-tracer_gb300/jni/dfpt_jni.c), compiled against a
stand-in jni.h and driven through a fake JNIEnv (tests/jni/): no JDK exists on either machine.

CPU: the shim compiles with warnings as errors, exports one function per native method of
CudaRendererKernel.java with the matching parameter count, and turns every failure of the core
into the Java exception the reference would throw, holding no critical section across other JNI
calls. GPU: a kernel created and driven through the shim (its frame tuner included) renders the
same image and selection buffer as the ctypes binding with the same seed and knobs, across a sun
toggle and a clear.
"""
import ctypes as C

import numpy as np
import pytest

import _jni


@pytest.fixture(scope="module")
def shim(tmp_path_factory, lib):
    return _jni.Shim(_jni.build(tmp_path_factory.mktemp("jni")))


def _scene(w=16, h=16):
    from dfpt import synthetic

    scene, sky, params, _ = synthetic.sphere_scene(0, w, h)
    return scene, sky, params


def test_every_native_method_has_its_jni_function(shim):
    java = _jni.java_natives()
    c = _jni.c_natives()
    assert set(java) == set(c), (set(java) ^ set(c))
    for name, types in java.items():
        assert c[name] == len(types) + 2, name  # JNIEnv* and jclass come first
        assert hasattr(shim.so, _jni.PREFIX + name)


def test_null_array_throws_null_pointer_exception(shim):
    scene, sky, _ = _scene()
    h = _jni.create(shim, scene, sky, 16, 16, 1, drop="camera")
    assert h == 0
    assert shim.exception() == ("java/lang/NullPointerException", "camera == null")
    assert shim.violations() == 0


def test_bad_resolution_throws_illegal_argument_exception(shim):
    scene, sky, _ = _scene()
    h = _jni.create(shim, scene, sky, 0, 16, 1)
    assert h == 0
    cls, msg = shim.exception()
    assert cls == "java/lang/IllegalArgumentException" and msg
    assert shim.violations() == 0  # the 14 arrays were released


def test_invalid_scene_throws_illegal_argument_exception(shim):
    scene, sky, _ = _scene()
    s = scene.copy()
    s.primitives[1] = 999  # a sphere offset past spheres[]
    assert _jni.create(shim, s, sky, 16, 16, 1) == 0
    assert shim.exception()[0] == "java/lang/IllegalArgumentException"
    assert shim.violations() == 0


def test_bad_sky_arrays_throw_before_any_device_work(shim):
    scene, sky, _ = _scene()
    arrays = [shim.array(getattr(scene, k)) for k in _jni.SCENE_ORDER]
    d, f, flags = _jni.sky_arrays(sky)
    assert shim.nativeCreate(*arrays, shim.array(d[:17]), shim.array(f), flags, 16, 16, 1) == 0
    assert shim.exception() == ("java/lang/IllegalArgumentException", "sky arrays must hold 18 doubles and 19 floats")


def test_calls_without_a_kernel_throw_illegal_state_exception(shim):
    shim.nativeRender(0, 1)
    assert shim.exception()[0] == "java/lang/IllegalStateException"
    shim.nativeTuneFrame(0, 8)
    assert shim.exception()[0] == "java/lang/IllegalStateException"
    img = np.zeros(16, np.uint8)
    shim.nativeReadBgra8(0, shim.array(img))
    assert shim.exception()[0] == "java/lang/IllegalStateException"
    shim.nativeDestroy(0)  # disposing twice is a no-op, as the Java side's handle check makes it
    assert shim.exception() is None


@pytest.mark.gpu
def test_shim_renders_what_the_c_abi_renders(shim):
    from dfpt.kernel import RendererKernel

    w, h, seed = 64, 48, 0x1234
    scene, sky, params = _scene(w, h)
    ref = RendererKernel(scene, sky, params)
    ref.update(w, h)
    ref.set_seed(seed)

    handle = _jni.create(shim, scene, sky, w, h, seed)
    assert handle != 0, shim.exception()
    ints, floats = _jni.param_arrays(ref.params)
    shim.nativeSetParams(handle, shim.array(ints), shim.array(floats))
    assert shim.exception() is None
    # CudaRendererKernel.update() ends with the frame tuner, which leaves film and streams as they were.
    shim.nativeTuneFrame(handle, 2)
    assert shim.exception() is None

    def frame_pair(frames):
        img = np.zeros(w * h * 4, np.uint8)
        for _ in range(frames):
            shim.nativeRender(handle, 1)  # CudaRendererKernel.execute(range)
            assert shim.exception() is None
            ref.execute(1)
        shim.nativeReadBgra8(handle, shim.array(img))
        assert shim.exception() is None and shim.violations() == 0
        return img, ref.get()

    def same_image(a, b):
        # Sun shadow contributions are added with float atomics: the order of the adds may move a
        # channel by one step of 8 bits.
        d = np.abs(a.astype(np.int16) - np.asarray(b).reshape(-1).astype(np.int16))
        assert d.max() <= 1 and (d > 0).mean() < 0.01, (d.max(), (d > 0).mean())

    a, b = frame_pair(4)
    same_image(a, b)
    offsets = np.zeros(w * h, np.int32)
    shim.nativeReadPrimitiveOffsets(handle, shim.array(offsets))
    assert shim.exception() is None
    np.testing.assert_array_equal(offsets, ref.primitive_offsets().reshape(-1))

    # toggleSun (the Java side flips its flag bit and pushes the sky) and clear().
    d, f, flags = _jni.sky_arrays(sky)
    shim.nativeSetSky(handle, shim.array(d), shim.array(f), flags & ~2)
    shim.nativeClear(handle)
    assert shim.exception() is None
    ref.toggle_sun()
    ref.clear()
    a, b = frame_pair(2)
    same_image(a, b)

    # A wrong image size is refused before any copy.
    shim.nativeReadBgra8(handle, shim.array(np.zeros(w * h * 4 - 4, np.uint8)))
    assert shim.exception()[0] == "java/lang/IllegalArgumentException"

    shim.nativeDestroy(handle)
    assert shim.exception() is None
    ref.dispose()
