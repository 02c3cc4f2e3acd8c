//! Raw declarations of include/ferrokmeans.h, one for one (same names, field
//! order and types). tests/test_rust_ffi_layout.py in the repository parses
//! both files and checks that they agree.
#![allow(non_camel_case_types)]

use core::ffi::{c_char, c_void};

pub const FK_OK: i32 = 0;
pub const FK_ERR_INVALID_PARAMETER: i32 = 1;
pub const FK_ERR_INSUFFICIENT_SAMPLES: i32 = 2;
pub const FK_ERR_SHAPE_MISMATCH: i32 = 3;
pub const FK_ERR_NUMERICAL_INSTABILITY: i32 = 4;
pub const FK_ERR_CUDA: i32 = 10;
pub const FK_ERR_OOM: i32 = 11;
pub const FK_ERR_TIMEOUT: i32 = 12;
pub const FK_ERR_UNSUPPORTED: i32 = 13;
pub const FK_ERR_NULL_POINTER: i32 = 14;

pub const FK_PRECISION_PLAIN: i32 = 0;
pub const FK_PRECISION_MIXED_BF16: i32 = 1;
pub const FK_PRECISION_MIXED_FP8: i32 = 2;

pub const FK_REDUCE_REFERENCE: i32 = 0;
pub const FK_REDUCE_F64: i32 = 1;

pub const FK_MB_INIT_KMEANS_PLUS_PLUS: i32 = 0;
pub const FK_MB_INIT_RANDOM: i32 = 1;

pub const FK_BISECT_LARGEST_CLUSTER: i32 = 0;
pub const FK_BISECT_LARGEST_SSE: i32 = 1;

#[repr(C)]
pub struct fk_ctx {
    _opaque: [u8; 0],
}

#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct fk_kmeans_params {
    pub n_clusters: i64,
    pub max_iter: i64,
    pub tol: f64,
    pub n_init: i64,
    pub random_state: u64,
    pub has_random_state: i32,
    pub precision: i32,
    pub draws: *const f64,
    pub n_draws: i64,
    pub collect_timing: i32,
    pub reserved: i32,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default)]
pub struct fk_fit_report {
    pub best_run: i64,
    pub iterations_total: i64,
    pub rows_assigned: i64,
    pub rows_rechecked: i64,
    pub rows_full_rescan: i64,
    pub rows_fp64: i64,
    pub rows_second_pass: i64,
    pub rows_few: i64,
    pub rows_exhaustive: i64,
    pub near_tie_rows: i64,
    pub ms_init: f64,
    pub ms_assign: f64,
    pub ms_contract: f64,
    pub ms_update: f64,
    pub ms_total: f64,
    pub precision_used: i32,
    pub reserved: i32,
    pub rows_moved: i64,
    pub updates_incremental: i64,
    pub count_iterations: i64,
    pub ms_count_pass: f64,
}

#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct fk_batch_problem {
    pub x: *const f32,
    pub n: i64,
    pub d: i64,
    pub n_clusters: i64,
    pub max_iter: i64,
    pub tol: f64,
    pub n_init: i64,
    pub random_state: u64,
    pub init: *const f32,
    pub centers_out: *mut f32,
    pub labels_out: *mut u64,
    pub inertia_out: *mut f32,
    pub n_iter_out: *mut i64,
    pub best_run_out: *mut i64,
}

#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct fk_batch_report {
    pub fits: i64,
    pub iterations_total: i64,
    pub graph_launches: i64,
    pub tuned_buckets: i64,
    pub bucket_variant: [i32; 20],
    pub ms_upload: f64,
    pub ms_init: f64,
    pub ms_tune: f64,
    pub ms_lloyd: f64,
    pub ms_download: f64,
    pub ms_total: f64,
    pub fit_inertia: *mut f64,
    pub fit_n_iter: *mut i64,
}

#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct fk_minibatch_params {
    pub n_clusters: i64,
    pub batch_size: i64,
    pub max_iter: i64,
    pub tol: f64,
    pub n_init: i64,
    pub random_state: u64,
    pub has_random_state: i32,
    pub init: i32,
}

#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct fk_bisecting_params {
    pub n_clusters: i64,
    pub max_iter: i64,
    pub n_init: i64,
    pub random_state: u64,
    pub has_random_state: i32,
    pub strategy: i32,
}

unsafe extern "C" {
    pub fn fk_ctx_create(out: *mut *mut fk_ctx, device: i32, cuda_stream: *mut c_void) -> i32;
    pub fn fk_ctx_destroy(ctx: *mut fk_ctx) -> i32;
    pub fn fk_last_error_message() -> *const c_char;
    pub fn fk_version() -> *const c_char;
    pub fn fk_debug_launch_count() -> u64;
    pub fn fk_kmeans_params_default(p: *mut fk_kmeans_params, n_clusters: i64);
    pub fn fk_draws_f64(seed: u64, count: i64, out: *mut f64) -> i32;
    pub fn fk_kmeans_fit_f64(ctx: *mut fk_ctx, x: *const f64, n: i64, d: i64, params: *const fk_kmeans_params,
                             init_centers: *const f64, centers_out: *mut f64, labels_out: *mut u64,
                             inertia_out: *mut f64, n_iter_out: *mut i64, report: *mut fk_fit_report) -> i32;
    pub fn fk_kmeans_fit_f32(ctx: *mut fk_ctx, x: *const f32, n: i64, d: i64, params: *const fk_kmeans_params,
                             init_centers: *const f32, centers_out: *mut f32, labels_out: *mut u64,
                             inertia_out: *mut f32, n_iter_out: *mut i64, report: *mut fk_fit_report) -> i32;
    pub fn fk_kmeans_fit_f32x64(ctx: *mut fk_ctx, x: *const f32, n: i64, d: i64, params: *const fk_kmeans_params,
                                init_centers: *const f64, centers_out: *mut f64, labels_out: *mut u64,
                                inertia_out: *mut f64, n_iter_out: *mut i64, report: *mut fk_fit_report) -> i32;
    pub fn fk_lloyd_step_f64(ctx: *mut fk_ctx, x: *const f64, n: i64, d: i64, centers_in: *const f64, k: i64,
                             precision: i32, labels_out: *mut u64, centers_out: *mut f64, inertia_out: *mut f64,
                             max_shift_out: *mut f64, report: *mut fk_fit_report) -> i32;
    pub fn fk_lloyd_step_f32(ctx: *mut fk_ctx, x: *const f32, n: i64, d: i64, centers_in: *const f32, k: i64,
                             precision: i32, labels_out: *mut u64, centers_out: *mut f32, inertia_out: *mut f32,
                             max_shift_out: *mut f32, report: *mut fk_fit_report) -> i32;
    pub fn fk_lloyd_step_f32x64(ctx: *mut fk_ctx, x: *const f32, n: i64, d: i64, centers_in: *const f64, k: i64,
                                precision: i32, labels_out: *mut u64, centers_out: *mut f64, inertia_out: *mut f64,
                                max_shift_out: *mut f64, report: *mut fk_fit_report) -> i32;
    pub fn fk_kmeans_predict_f64(ctx: *mut fk_ctx, centers: *const f64, k: i64, d_fit: i64, x: *const f64, n: i64,
                                 d: i64, precision: i32, labels_out: *mut u64) -> i32;
    pub fn fk_kmeans_predict_f32(ctx: *mut fk_ctx, centers: *const f32, k: i64, d_fit: i64, x: *const f32, n: i64,
                                 d: i64, precision: i32, labels_out: *mut u64) -> i32;
    pub fn fk_kmeans_predict_f32x64(ctx: *mut fk_ctx, centers: *const f64, k: i64, d_fit: i64, x: *const f32,
                                    n: i64, d: i64, precision: i32, labels_out: *mut u64) -> i32;
    pub fn fk_kmeans_transform_f64(ctx: *mut fk_ctx, centers: *const f64, k: i64, d_fit: i64, x: *const f64, n: i64,
                                   d: i64, out: *mut f64) -> i32;
    pub fn fk_kmeans_transform_f32(ctx: *mut fk_ctx, centers: *const f32, k: i64, d_fit: i64, x: *const f32, n: i64,
                                   d: i64, out: *mut f32) -> i32;
    pub fn fk_kmeans_plus_plus_f64(ctx: *mut fk_ctx, x: *const f64, n: i64, d: i64, k: i64, draws: *const f64,
                                   n_draws: i64, seed: u64, centers_out: *mut f64, draws_used_out: *mut i64) -> i32;
    pub fn fk_kmeans_plus_plus_f32(ctx: *mut fk_ctx, x: *const f32, n: i64, d: i64, k: i64, draws: *const f64,
                                   n_draws: i64, seed: u64, centers_out: *mut f32, draws_used_out: *mut i64) -> i32;
    pub fn fk_kmeans_score_f64_noalloc(x: *const f64, n: i64, d: i64, centers: *const f64, k: i64,
                                       labels_out: *mut u64, inertia_out: *mut f64, cuda_stream: *mut c_void) -> i32;
    pub fn fk_kmeans_fit_batched_f32(ctx: *mut fk_ctx, problems: *mut fk_batch_problem, n_problems: i64,
                                     reduction: i32, report: *mut fk_batch_report) -> i32;
    pub fn fk_minibatch_params_default(p: *mut fk_minibatch_params, n_clusters: i64);
    pub fn fk_minibatch_fit_f64(ctx: *mut fk_ctx, x: *const f64, n: i64, d: i64, params: *const fk_minibatch_params,
                                init_centers: *const f64, centers_out: *mut f64, labels_out: *mut u64,
                                inertia_out: *mut f64, n_iter_out: *mut i64, best_run_out: *mut i64,
                                report: *mut fk_fit_report) -> i32;
    pub fn fk_minibatch_fit_f32(ctx: *mut fk_ctx, x: *const f32, n: i64, d: i64, params: *const fk_minibatch_params,
                                init_centers: *const f32, centers_out: *mut f32, labels_out: *mut u64,
                                inertia_out: *mut f32, n_iter_out: *mut i64, best_run_out: *mut i64,
                                report: *mut fk_fit_report) -> i32;
    pub fn fk_bisecting_params_default(p: *mut fk_bisecting_params, n_clusters: i64);
    pub fn fk_bisecting_fit_f64(ctx: *mut fk_ctx, x: *const f64, n: i64, d: i64, params: *const fk_bisecting_params,
                                centers_out: *mut f64, labels_out: *mut i64, inertia_out: *mut f64,
                                n_clusters_out: *mut i64) -> i32;
    pub fn fk_bisecting_fit_f32(ctx: *mut fk_ctx, x: *const f32, n: i64, d: i64, params: *const fk_bisecting_params,
                                centers_out: *mut f32, labels_out: *mut i64, inertia_out: *mut f32,
                                n_clusters_out: *mut i64) -> i32;
    pub fn fk_minibatch_batch_indices(seed: u64, pos: i64, n: i64, batch_size: i64, iters: i64, out: *mut i64)
        -> i32;
    pub fn fk_debug_measure_peaks(ctx: *mut fk_ctx, out: *mut f64) -> i32;
    pub fn fk_debug_measure_tc_peaks(ctx: *mut fk_ctx, out: *mut f64) -> i32;
    pub fn fk_debug_tc_probe(ctx: *mut fk_ctx, x_dev: *const f32, n: i64, d: i64, c_dev: *const f64, k: i64,
                             precision: i32, dump: *mut f32, xq: *mut c_void, cq: *mut c_void, aug: *mut u16,
                             xaug: *mut u16, top: *mut c_void, plan: *mut i32) -> i32;
    pub fn fk_debug_tc_plan(n: i64, d: i64, k: i64, precision: i32, topk: i32, num_sms: i32, out: *mut i64) -> i32;
}
