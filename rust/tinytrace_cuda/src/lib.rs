//! Safe wrapper over `tinytrace_cuda_sys` with the operations tinytrace's `Renderer` and
//! `Scene` perform through `tinytrace_backend::Context` on the rendering hot path.
//!
//! A maintainer swaps the backend calls of `src/lib.rs`, `src/scene.rs`,
//! `src/integrate/mod.rs` and `src/post_process/mod.rs` for the methods below, keeping the
//! public `Renderer` / `Scene` / `Camera` / `Config` API of the reference unchanged:
//!
//! | reference call site | method |
//! |---|---|
//! | `Context::new` (src/lib.rs:64) | [`Context::new`] |
//! | `create_render_target` (src/lib.rs:213-226) | [`Context::create_render_target`] |
//! | `Scene::new` buffer uploads and BLAS/TLAS builds (src/scene.rs:66-171) | [`Context::create_scene`] |
//! | `clear_resources_with_lifetime(Lifetime::Scene)` (src/lib.rs:98-99) | [`Context::clear_lifetime`] |
//! | `Integrator::integrate` (src/integrate/mod.rs:39-61) | [`Context::render`] |
//! | `download` in `render_to_texture` (src/lib.rs:201-210) | [`Context::download`] |
//! | `PostProcess::run` + `present` (src/lib.rs:180-199) | [`Context::tonemap`], [`Context::advance_frame`] |
//! | `Renderer::timings` (src/lib.rs:167-178) | [`Context::timings`] |
//! | `Context::frame_index` (src/lib.rs:130) | [`Context::frame_index`] |
//!
//! Errors carry the status code and the library's message; nothing panics across the FFI.

use std::ffi::CStr;
use std::fmt;
use std::ptr;
use std::time::Duration;

pub use tinytrace_cuda_sys as sys;
use sys::*;

/// A failed call: the status code (TT_ERR_*) and `tt_last_error`'s message.
#[derive(Debug, Clone)]
pub struct Error {
    pub code: i32,
    pub message: String,
}

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "tinytrace_cuda error {}: {}", self.code, self.message)
    }
}

impl std::error::Error for Error {}

fn check(status: i32) -> Result<(), Error> {
    if status == TT_OK {
        return Ok(());
    }
    // SAFETY: tt_last_error returns a thread-local NUL-terminated string (or null).
    let message = unsafe {
        let p = tt_last_error();
        if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
    };
    Err(Error { code: status, message })
}

/// Device handle of a render target or scene; invalid after its lifetime is cleared (calls
/// with it then fail with TT_ERR_BAD_HANDLE instead of panicking as the reference does).
#[derive(Debug, Clone, Copy, PartialEq, Eq)]
pub struct Handle(pub tt_handle);

/// `Timings` of src/lib.rs:228-232.
#[derive(Debug, Clone, Copy)]
pub struct Timings {
    pub integrate: Duration,
    pub post_process: Duration,
}

/// The borrowed arrays of one scene, laid out as the reference lays out `asset::Scene` and the
/// instances / emissive triangles that `Scene::new` derives from its node tree.
pub struct SceneArrays<'a> {
    pub positions: &'a [[i16; 3]],
    pub indices: &'a [u32],
    pub vertices: &'a [tt_vertex],
    pub materials: &'a [tt_material],
    pub meshes: &'a [tt_mesh],
    pub instances: &'a [tt_instance],
    pub emissive_triangles: &'a [tt_emissive_triangle],
    pub textures: &'a [tt_texture],
}

/// One GPU context: a CUDA stream and the device resources it owns.  Used by one thread at a
/// time, like the reference's `Renderer` (`&mut self` throughout).
pub struct Context {
    raw: *mut tt_context,
}

impl Context {
    pub fn new(device: i32) -> Result<Self, Error> {
        let mut raw = ptr::null_mut();
        // SAFETY: `raw` is a valid out-pointer.
        check(unsafe { tt_context_create(device, &mut raw) })?;
        Ok(Context { raw })
    }

    pub fn frame_index(&self) -> Result<u64, Error> {
        let mut v = 0u64;
        check(unsafe { tt_frame_index(self.raw, &mut v) })?;
        Ok(v)
    }

    pub fn advance_frame(&mut self) -> Result<(), Error> {
        check(unsafe { tt_advance_frame(self.raw) })
    }

    pub fn clear_lifetime(&mut self, lifetime: u32) -> Result<(), Error> {
        check(unsafe { tt_clear_lifetime(self.raw, lifetime) })
    }

    pub fn set_option(&mut self, option: u32, value: u64) -> Result<(), Error> {
        check(unsafe { tt_set_option(self.raw, option, value) })
    }

    /// The RGBA32F render target (surface lifetime).
    pub fn create_render_target(&mut self, width: u32, height: u32) -> Result<Handle, Error> {
        let mut h = 0;
        check(unsafe { tt_image_create(self.raw, TT_LIFETIME_SURFACE, width, height, &mut h) })?;
        Ok(Handle(h))
    }

    /// Uploads the scene arrays and builds the acceleration structure (scene lifetime).
    pub fn create_scene(&mut self, s: &SceneArrays<'_>) -> Result<Handle, Error> {
        let desc = tt_scene_desc {
            positions: s.positions.as_ptr() as *const i16,
            position_count: s.positions.len() as u64,
            indices: s.indices.as_ptr(),
            index_count: s.indices.len() as u64,
            vertices: s.vertices.as_ptr(),
            vertex_count: s.vertices.len() as u64,
            materials: s.materials.as_ptr(),
            material_count: s.materials.len() as u32,
            mesh_count: s.meshes.len() as u32,
            meshes: s.meshes.as_ptr(),
            instances: s.instances.as_ptr(),
            instance_count: s.instances.len() as u32,
            emissive_triangle_count: s.emissive_triangles.len() as u32,
            emissive_triangles: s.emissive_triangles.as_ptr(),
            textures: s.textures.as_ptr(),
            texture_count: s.textures.len() as u32,
            reserved: 0,
        };
        let mut h = 0;
        // SAFETY: the arrays outlive the call; the library copies them before it returns.
        check(unsafe { tt_scene_create(self.raw, &desc, &mut h) })?;
        Ok(Handle(h))
    }

    /// New instance transforms of a scene (the TLAS update); the structure is refitted.
    pub fn update_instances(&mut self, scene: Handle, instances: &[tt_instance]) -> Result<(), Error> {
        check(unsafe { tt_scene_update_instances(self.raw, scene.0, instances.as_ptr(), instances.len() as u32) })
    }

    /// One frame of the path tracer into `target` with the reference's accumulation rule.
    pub fn render(&mut self, scene: Handle, constants: &tt_constants, target: Handle) -> Result<(), Error> {
        check(unsafe { tt_render(self.raw, scene.0, constants, target.0) })
    }

    /// One ReSTIR DI frame (direct light at the primary hit, one sample per pixel).
    pub fn render_restir(&mut self, scene: Handle, constants: &tt_constants, target: Handle) -> Result<(), Error> {
        check(unsafe { tt_render_restir(self.raw, scene.0, constants, target.0) })
    }

    /// The render target as RGBA32F, row-major (width * height * 4 floats).
    pub fn download(&mut self, target: Handle, out: &mut [f32]) -> Result<(), Error> {
        check(unsafe { tt_image_download(self.raw, target.0, out.as_mut_ptr(), (out.len() * 4) as u64) })
    }

    /// The display pass (tonemap, RGBA8) into a host pixel buffer of width * height * 4 bytes.
    pub fn tonemap(&mut self, target: Handle, constants: &tt_constants, out: &mut [u8]) -> Result<(), Error> {
        check(unsafe {
            tt_tonemap(self.raw, target.0, constants, TT_FORMAT_RGBA8_UNORM, out.as_mut_ptr().cast(), out.len() as u64)
        })
    }

    pub fn timings(&mut self) -> Result<Timings, Error> {
        let mut t = tt_timings::default();
        check(unsafe { tt_timings_get(self.raw, &mut t) })?;
        Ok(Timings {
            integrate: Duration::from_nanos(t.integrate_ns),
            post_process: Duration::from_nanos(t.post_process_ns),
        })
    }

    /// Tunes the integrator for this scene and camera with a few-sample copy of the frame.
    pub fn autotune(&mut self, scene: Handle, constants: &tt_constants, target: Handle) -> Result<tt_tune_result, Error> {
        let mut r = tt_tune_result::default();
        check(unsafe { tt_autotune(self.raw, scene.0, constants, target.0, &mut r) })?;
        Ok(r)
    }

    pub fn wait_until_idle(&mut self) -> Result<(), Error> {
        check(unsafe { tt_synchronize(self.raw) })
    }

    /// The raw context, for the entry points this wrapper does not cover.
    pub fn as_raw(&self) -> *mut tt_context {
        self.raw
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        // SAFETY: `raw` came from tt_context_create and is destroyed once.
        unsafe {
            tt_context_destroy(self.raw);
        }
    }
}
