//! The GI pass as a stage of the reference renderer: `GiStage` implements
//! the renderer's `RenderStage<AppState>` trait (reference: src/app.rs:3-7)
//! on top of librc.so.  `update` uploads the frame's emitters (the call site
//! is src/window/app.rs:131), `render` enqueues every cascade and the
//! cascade-0 fluence (src/window/app.rs:246-248), `resize` has nothing to
//! rebuild because the GI grid does not follow the window
//! (src/window/app.rs:109).  Errors are logged with the engine's message;
//! nothing aborts, where the reference would panic.
pub mod ffi;

use crate::app::{AppState, RenderStage};
use ffi::*;
use std::ffi::CStr;

/// Logs the engine's message for a failed call and passes the status on.
fn check(s: rc_status) -> rc_status {
    if s != RC_OK {
        let msg = unsafe { CStr::from_ptr(rc_last_error()) }.to_string_lossy();
        log::error!("GI stage: {}", msg);
    }
    s
}

pub struct GiStage {
    ctx: *mut rc_context,
    params: rc_params,
    spheres: Vec<rc_sphere>,
    fluence: Vec<f32>,
}

impl GiStage {
    /// A cubic grid of `grid` voxels with `cascades` cascades, the static
    /// scene given as boxes, and the moving emitters.
    pub fn new(grid: i32, cascades: i32, boxes: &[rc_box], spheres: Vec<rc_sphere>) -> Option<Self> {
        let mut params = rc_params::default();
        let mut ctx = std::ptr::null_mut();
        unsafe {
            if check(rc_params_default(&mut params, grid, cascades)) != RC_OK
                || check(rc_create(&params, 0, &mut ctx)) != RC_OK
            {
                return None;
            }
            if check(rc_scene_set_boxes(ctx, boxes.as_ptr(), boxes.len() as i32)) != RC_OK {
                rc_destroy(ctx);
                return None;
            }
        }
        let n = unsafe { rc_fluence_elems(&params) } as usize;
        Some(Self { ctx, params, spheres, fluence: vec![0.0; n] })
    }

    /// Switches the far cascades to the learned form (neural radiance cache).
    pub fn enable_cache(&mut self) -> bool {
        let mut p = rc_nrc_params::default();
        unsafe { check(rc_nrc_params_default(&mut p)) == RC_OK && check(rc_nrc_enable(self.ctx, &p)) == RC_OK }
    }

    /// Cascade-0 fluence of the last solve, RGB per probe (host copy).
    pub fn fluence(&mut self) -> &[f32] {
        unsafe {
            check(rc_get_fluence(self.ctx, self.fluence.as_mut_ptr(), self.fluence.len() as i64, RC_MEM_HOST));
        }
        &self.fluence
    }

    /// Device address of the fluence for a consumer on the same GPU.
    pub fn fluence_device_ptr(&self) -> *const f32 {
        let mut p = std::ptr::null();
        unsafe { check(rc_fluence_device_ptr(self.ctx, &mut p)) };
        p
    }

    pub fn params(&self) -> &rc_params {
        &self.params
    }

    /// Emitters for the next frame: advanced along their paths by the engine's
    /// own rule (reflected at the grid walls).
    pub fn advance(&mut self, frames: i32) {
        unsafe {
            check(rc_spheres_advance(self.spheres.as_mut_ptr(), self.spheres.len() as i32,
                                     self.params.grid.as_ptr(), frames));
        }
    }
}

impl RenderStage<AppState> for GiStage {
    fn update(&mut self, _state: &AppState, _queue: &wgpu::Queue) {
        unsafe { check(rc_scene_set_spheres(self.ctx, self.spheres.as_ptr(), self.spheres.len() as i32)) };
    }

    fn render(&self, _state: &mut AppState, _view: &wgpu::TextureView, _encoder: &mut wgpu::CommandEncoder) {
        unsafe { check(rc_solve(self.ctx, std::ptr::null_mut())) };
    }

    fn resize(&mut self, _device: &wgpu::Device, _config: &wgpu::SurfaceConfiguration) {}
}

impl Drop for GiStage {
    fn drop(&mut self) {
        unsafe {
            rc_destroy(self.ctx);
        }
    }
}
