"""Host-side RendererKernel behaviour that needs no GPU: the setters, getters, toggles, predicates
and change flag of AbstractRendererKernel / AbstractKernel
(src/main/java/org/dayflower/pathtracer/kernel/AbstractRendererKernel.java:238-690,
AbstractKernel.java:205-295). No handle is created (update() is not called), so nothing is pushed
to a device."""
import math

import pytest

from dfpt import kernel as K
from dfpt import synthetic


@pytest.fixture()
def rk():
    scene, sky, params, _ = synthetic.sphere_scene(0, 8, 8)
    return K.RendererKernel(scene, sky, params)


def test_setters_mark_changes_and_ignore_unknown_values(rk):
    assert not rk.has_changed()
    rk.set_renderer_type(rk.get_renderer_type())  # same value: no change (AbstractRendererKernel.java:413)
    assert not rk.has_changed()
    rk.set_renderer_type(K.RENDERER_TYPE_RAY_CASTER)
    assert rk.has_changed() and rk.is_renderer_type_ray_caster()
    rk.set_changed(False)
    rk.set_renderer_type(99)  # unknown: ignored
    rk.set_shader_type(7)
    rk.set_tone_mapper_type(0)
    rk.set_renderer_normal_mapping(2)
    rk.set_renderer_wireframes(-1)
    assert not rk.has_changed() and rk.get_renderer_type() == K.RENDERER_TYPE_RAY_CASTER
    rk.set_renderer_ao_maximum_distance(rk.get_renderer_ao_maximum_distance())
    assert not rk.has_changed()
    rk.set_renderer_ao_maximum_distance(123.5)
    assert rk.has_changed() and rk.get_renderer_ao_maximum_distance() == 123.5


def test_float_compare_semantics(rk):
    rk.set_tone_mapper_exposure(float("nan"))
    rk.set_changed(False)
    rk.set_tone_mapper_exposure(float("nan"))  # Float.compare(NaN, NaN) == 0
    assert not rk.has_changed() and math.isnan(rk.get_tone_mapper_exposure())
    rk.set_tone_mapper_exposure(0.0)
    rk.set_changed(False)
    rk.set_tone_mapper_exposure(-0.0)  # Float.compare(0.0, -0.0) != 0
    assert rk.has_changed() and math.copysign(1.0, rk.get_tone_mapper_exposure()) < 0


def test_toggles_cycle_as_the_reference(rk):
    rk.set_renderer_type(K.RENDERER_TYPE_AMBIENT_OCCLUSION)
    seen = []
    for _ in range(6):
        rk.toggle_renderer_type()
        seen.append(rk.get_renderer_type())
    assert seen == [K.RENDERER_TYPE_PATH_TRACER, K.RENDERER_TYPE_RAY_CASTER, K.RENDERER_TYPE_RAY_MARCHER,
                    K.RENDERER_TYPE_RAY_TRACER, K.RENDERER_TYPE_SURFACE_NORMALS, K.RENDERER_TYPE_AMBIENT_OCCLUSION]
    predicates = [rk.is_renderer_type_ambient_occlusion, rk.is_renderer_type_path_tracer, rk.is_renderer_type_ray_caster,
                  rk.is_renderer_type_ray_marcher, rk.is_renderer_type_ray_tracer, rk.is_renderer_type_surface_normals]
    for t in range(1, 7):
        rk.set_renderer_type(t)
        assert [p() for p in predicates] == [i + 1 == t for i in range(6)]
    rk.set_shader_type(K.SHADER_TYPE_FLAT)
    rk.toggle_shader_type()
    assert rk.get_shader_type() == K.SHADER_TYPE_GOURAUD
    rk.toggle_shader_type()
    assert rk.get_shader_type() == K.SHADER_TYPE_FLAT
    for toggle, get in ((rk.toggle_renderer_normal_mapping, rk.get_renderer_normal_mapping),
                        (rk.toggle_renderer_wireframes, rk.get_renderer_wireframes)):
        before = get()
        rk.set_changed(False)
        toggle()
        assert get() == 1 - before and rk.has_changed()
        toggle()
        assert get() == before


def test_global_noise_setters_mark_nothing(rk):
    rk.set_global_amplitude(0.25)
    rk.set_global_frequency(2.0)
    rk.set_global_gain(0.75)
    rk.set_global_lacunarity(3.0)
    rk.set_global_octaves(4)
    assert not rk.has_changed()  # AbstractKernel's setters have no change flag
    assert (rk.get_global_amplitude(), rk.get_global_frequency(), rk.get_global_gain(), rk.get_global_lacunarity(),
            rk.get_global_octaves()) == (0.25, 2.0, 0.75, 3.0, 4)


def test_scene_accessors(rk):
    assert rk.get_compiled_scene() is rk.compiled
    assert rk.get_sky() is rk.sky
    assert rk.get_camera().shape == (19,)


def test_sky_and_sun_toggles_mark_changes(rk):
    sky0, sun0 = rk.get_sky().raw.is_sky_active, rk.get_sky().raw.is_sun_active
    rk.toggle_sky()
    assert rk.has_changed() and rk.get_sky().raw.is_sky_active == 1 - sky0
    rk.set_changed(False)
    rk.toggle_sun()
    assert rk.has_changed() and rk.get_sky().raw.is_sun_active == 1 - sun0


def test_primitive_material_toggle_cycles_the_selected_surface(rk):
    from dfpt.scene import CLEAR_COAT, GLASS, LAMBERTIAN, PHONG, REFLECTION

    rk.toggle_primitive_material()  # nothing selected: no change (GPURendererKernel.togglePrimitiveMaterial)
    assert not rk.has_changed()
    off = 3  # the second primitive's offset in the primitives array
    rk._selected_primitive_offset = off
    so = int(rk.compiled.primitives[off + 2])
    order = [CLEAR_COAT, GLASS, LAMBERTIAN, PHONG, REFLECTION]
    first = int(rk.compiled.surfaces[so])
    for k in range(1, 6):
        rk.toggle_primitive_material()
        assert int(rk.compiled.surfaces[so]) == order[(first - 1 + k) % 5]
    assert rk.has_changed()
