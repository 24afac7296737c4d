"""Camera, light and parameter-block set-up for the raymarcher.

Restates the reference's host-side math that fills the raymarch UBOs:
  * Camera::recalculate_view_matrix / recalculate_projection_matrix
    (src/vkhr/scene_graph/camera.cc:225-249): glm::lookAt (right-handed),
    glm::perspective with depth in [0, 1] (GLM_FORCE_DEPTH_ZERO_TO_ONE,
    camera.cc:4), then projection[1][1] *= -1 for Vulkan (camera.cc:229);
    near 1, far 10000, field of view pi/4 (include/vkhr/scene_graph/camera.hh:92-101);
  * the directional light's origin, look_at + normalize(direction) * camera
    distance (src/vkhr/scene_graph.cc:124-127, light_source.cc:131-134);
  * the Params UBO defaults of Interface::Parameters
    (include/vkhr/rasterizer/interface.hh:86-112): iso 0.115, 1024 steps,
    AO radius 2.5, exponent 10, clamp 0.16, LoD distances 400/800;
  * hair_exponent 80 (src/vkhr/rasterizer/hair_style.cc:59).
Matrices are column-major float32[16], the memory layout of glm::mat4.
"""
import numpy as np

from . import _abi


def look_at(eye, center, up):
    eye, center, up = (np.asarray(a, dtype=np.float64) for a in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)  # m[col][row] as glm stores it
    m[0][0], m[1][0], m[2][0] = s
    m[0][1], m[1][1], m[2][1] = u
    m[0][2], m[1][2], m[2][2] = -f
    m[3][0] = -np.dot(s, eye)
    m[3][1] = -np.dot(u, eye)
    m[3][2] = np.dot(f, eye)
    return m


def perspective_zo(fovy, aspect, znear, zfar):
    t = np.tan(fovy / 2.0)
    m = np.zeros((4, 4))
    m[0][0] = 1.0 / (aspect * t)
    m[1][1] = 1.0 / t
    m[2][2] = zfar / (znear - zfar)
    m[2][3] = -1.0
    m[3][2] = -(zfar * znear) / (zfar - znear)
    return m


def colmajor(m):
    """glm::mat4 memory (m[col][row]) as a flat float32[16]."""
    return np.asarray(m, dtype=np.float32).reshape(16)


def make_params(bounds, resolution, width, height, camera_distance=4.0, fov_degrees=45.0,
                view_direction=(0.0, 0.0, 1.0), light_direction=(1.0, 2.0, 1.0),
                light_intensity=(0.430, 0.380, 0.280), raycast_steps=512.0, isosurface=0.115,
                hair_color=(0.40, 0.32, 0.24), hair_alpha=0.5, hair_exponent=80.0,
                shading_model=_abi.SHADING_KAJIYA_KAY, deep_shadows_on=1, occlusion_radius=2.5,
                ao_exponent=10.0, ao_max=0.16, renderer=_abi.RENDERER_RAYMARCHER, shadow_steps=0.0, kd=1.0,
                density_format=_abi.DENSITY_U8_UNORM, tangent_format=_abi.TANGENT_I8_SNORM, target=None,
                spec_exponent2=0.0, spec_shift=(0.0, 0.0), ao_directions=0):
    """Reference-semantics raymarch parameters for a style with AABB `bounds`.

    The camera looks at the AABB centre (or `target`) from `camera_distance`
    along `view_direction`, up = +y; the light and intensity default to the
    reference's ponytail scene (share/scenes/ponytail.vkhr: direction
    (1, 2, 1), intensity (0.43, 0.38, 0.28)).  spec_exponent2, spec_shift and
    ao_directions are the extension knobs of vkhr_raymarch_params (a second,
    hair-coloured specular lobe, tangent shifts per lobe, directional AO);
    their defaults give the reference's shading.
    """
    p = _abi.RaymarchParams()
    p.width, p.height = int(width), int(height)
    o = np.array(bounds.origin, dtype=np.float64)
    s = np.array(bounds.size, dtype=np.float64)
    center = o + 0.5 * s if target is None else np.asarray(target, dtype=np.float64)
    vd = np.asarray(view_direction, dtype=np.float64)
    vd = vd / np.linalg.norm(vd)
    eye = (center + camera_distance * vd).astype(np.float32).astype(np.float64)
    view = look_at(eye, center, (0.0, 1.0, 0.0))
    proj = perspective_zo(np.deg2rad(fov_degrees), width / float(height), 1.0, 10000.0)
    proj[1][1] *= -1.0
    p.view[:] = colmajor(view).tolist()
    p.projection[:] = colmajor(proj).tolist()
    p.camera_position[:] = eye.astype(np.float32).tolist()
    dist = float(np.linalg.norm(center - eye))
    p.look_at_distance = dist
    ld = np.asarray(light_direction, dtype=np.float64)
    ld = ld / np.linalg.norm(ld)
    p.light_origin[:] = (center + ld * dist).astype(np.float32).tolist()
    p.light_intensity[:] = list(light_intensity)
    p.volume_bounds = bounds
    p.volume_resolution[:] = [int(r) for r in resolution]
    p.hair_color[:] = list(hair_color)
    p.hair_alpha = hair_alpha
    p.hair_exponent = hair_exponent
    p.shading_model = shading_model
    p.deep_shadows_on = deep_shadows_on
    p.isosurface = isosurface
    p.raycast_steps = raycast_steps
    p.occlusion_radius = occlusion_radius
    p.ao_exponent = ao_exponent
    p.ao_max = ao_max
    p.magnified_distance = 400.0
    p.renderer = renderer
    p.minified_distance = 800.0
    p.shadow_thickness = 11.0
    p.ao_kernel_size = 2.0
    p.shadow_steps = shadow_steps
    p.kd = kd
    p.density_format = density_format
    p.tangent_format = tangent_format
    p.spec_exponent2 = spec_exponent2
    p.spec_shift[:] = [float(x) for x in spec_shift]
    p.ao_directions = int(ao_directions)
    return p


# The shading the workloads name: Kajiya-Kay with kd 0.4, specular exponents
# 80 / 8 and tangent shifts +0.1 / -0.1.
CONFIG_SHADING = {"kd": 0.4, "hair_exponent": 80.0, "spec_exponent2": 8.0, "spec_shift": (0.1, -0.1)}

