//! GB300 (sm_103a) back end of ferrolearn-cluster's KMeans Lloyd path.
//!
//! The kernels are the hand-written CUDA of this repository
//! (ferrolearn_gb300/csrc, compiled by build.rs with nvcc for sm_103a); this
//! crate binds their C ABI (include/ferrokmeans.h, declared in [`ffi`]) and
//! exposes it in ferrolearn's own terms:
//!
//! * [`CudaKMeans`] / [`FittedCudaKMeans`]: the builder and fitted model of
//!   `ferrolearn_cluster::KMeans<F>` (kmeans.rs:55-156: same fields,
//!   defaults, builders and getters), implementing ferrolearn-core's `Fit`,
//!   `Predict` and `Transform` (traits.rs:83-157) for `F = f32` and `f64`,
//!   plus the tensor-core precisions for `KMeans<f64>` on f32 storage.
//! * [`fit_lloyd`], [`predict_nearest`], [`transform_distances`]: the hooks
//!   `impl Fit for KMeans<F>` (kmeans.rs:403-513), `Predict` (:528-553) and
//!   `Transform` (:555-618) call when ferrolearn-cluster is built with its
//!   `cuda` feature. `SpectralClustering::fit` (spectral.rs:283-289) then
//!   reaches the GPU through its KMeans call with no change of its own.
//!
//! Errors are ferrolearn's `FerroError`, one-to-one with the library's
//! status codes; failures of the CUDA side itself (no device, out of memory,
//! a bounded device wait that gave up, an unsupported shape) become
//! `NumericalInstability` with the library's message.
//!
//! Not compiled in the repository's own build (there is no Rust toolchain
//! there); the layout of [`ffi`] is checked against the header by a test.

pub mod ffi;

use core::ffi::CStr;
use core::ptr::{null, null_mut};
use std::cell::RefCell;

use ferrolearn_core::{FerroError, Fit, Predict, Transform};
use ndarray::{Array1, Array2};
use num_traits::Float;

/// Arithmetic of the distance contraction (ffi::FK_PRECISION_*). The labels
/// are those of the FP64 direct form in every case.
#[derive(Debug, Clone, Copy, PartialEq, Eq, Default)]
pub enum Precision {
    /// Direct-form distances in F on CUDA cores, bit-identical to kmeans.rs.
    #[default]
    Plain,
    /// BF16 tcgen05 contraction with the exact FP64 re-check (f64 model, f32 rows).
    MixedBf16,
    /// FP8 E4M3 contraction with per-row scales and the same re-check.
    MixedFp8,
}

impl Precision {
    fn code(self) -> i32 {
        match self {
            Precision::Plain => ffi::FK_PRECISION_PLAIN,
            Precision::MixedBf16 => ffi::FK_PRECISION_MIXED_BF16,
            Precision::MixedFp8 => ffi::FK_PRECISION_MIXED_FP8,
        }
    }
}

/// One GPU and one CUDA stream, with the device buffers the library keeps
/// across calls. The library wants one context per host thread.
pub struct Context {
    raw: *mut ffi::fk_ctx,
}

// A context may move to another thread; it is never used from two at once.
unsafe impl Send for Context {}

impl Context {
    /// A context on `device` with its own non-blocking stream.
    pub fn new(device: i32) -> Result<Self, FerroError> {
        let mut raw = null_mut();
        let st = unsafe { ffi::fk_ctx_create(&mut raw, device, null_mut()) };
        check(st, &Shape::default(), "creating a GPU context")?;
        Ok(Self { raw })
    }

    /// The raw handle, for the ffi functions.
    pub fn as_ptr(&self) -> *mut ffi::fk_ctx {
        self.raw
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe {
            ffi::fk_ctx_destroy(self.raw);
        }
    }
}

thread_local! {
    static THREAD_CTX: RefCell<Option<Context>> = const { RefCell::new(None) };
}

/// Runs f with this thread's context (on device 0, created on first use).
fn with_ctx<R>(f: impl FnOnce(*mut ffi::fk_ctx) -> Result<R, FerroError>) -> Result<R, FerroError> {
    THREAD_CTX.with(|cell| {
        let mut slot = cell.borrow_mut();
        if slot.is_none() {
            *slot = Some(Context::new(0)?);
        }
        f(slot.as_ref().map(Context::as_ptr).unwrap_or(null_mut()))
    })
}

fn last_error() -> String {
    unsafe {
        let p = ffi::fk_last_error_message();
        if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
    }
}

/// What the caller knows about a call's shapes, for the error variants.
#[derive(Default)]
struct Shape {
    k: usize,
    n: usize,
    d_fit: usize,
    d: usize,
}

fn check(st: i32, shape: &Shape, context: &str) -> Result<(), FerroError> {
    if st == ffi::FK_OK {
        return Ok(());
    }
    let msg = last_error();
    Err(match st {
        ffi::FK_ERR_INVALID_PARAMETER => {
            // "Invalid parameter `name`: reason"
            let name = msg.split('`').nth(1).unwrap_or("").to_string();
            let reason = msg.split_once("`: ").map(|(_, r)| r.to_string()).unwrap_or_else(|| msg.clone());
            FerroError::InvalidParameter { name, reason }
        }
        ffi::FK_ERR_INSUFFICIENT_SAMPLES => FerroError::InsufficientSamples {
            required: shape.k,
            actual: shape.n,
            context: context.to_string(),
        },
        ffi::FK_ERR_SHAPE_MISMATCH => FerroError::ShapeMismatch {
            expected: vec![shape.d_fit],
            actual: vec![shape.d],
            context: context.to_string(),
        },
        ffi::FK_ERR_NUMERICAL_INSTABILITY => FerroError::NumericalInstability { message: msg },
        _ => FerroError::NumericalInstability { message: format!("GPU back end, status {st} ({context}): {msg}") },
    })
}

/// The floating-point types with a GPU path (the reference's `F`).
pub trait GpuFloat: Float + Send + Sync + 'static {
    /// fk_kmeans_fit_f64 / _f32.
    ///
    /// # Safety
    /// The pointers must be valid for the sizes the header states.
    #[allow(clippy::too_many_arguments)]
    unsafe fn fit_raw(ctx: *mut ffi::fk_ctx, x: *const Self, n: i64, d: i64, p: *const ffi::fk_kmeans_params,
                      init: *const Self, centers: *mut Self, labels: *mut u64, inertia: *mut Self,
                      n_iter: *mut i64, report: *mut ffi::fk_fit_report) -> i32;
    /// fk_kmeans_predict_f64 / _f32.
    ///
    /// # Safety
    /// The pointers must be valid for the sizes the header states.
    #[allow(clippy::too_many_arguments)]
    unsafe fn predict_raw(ctx: *mut ffi::fk_ctx, c: *const Self, k: i64, d_fit: i64, x: *const Self, n: i64,
                          d: i64, labels: *mut u64) -> i32;
    /// fk_kmeans_transform_f64 / _f32.
    ///
    /// # Safety
    /// The pointers must be valid for the sizes the header states.
    #[allow(clippy::too_many_arguments)]
    unsafe fn transform_raw(ctx: *mut ffi::fk_ctx, c: *const Self, k: i64, d_fit: i64, x: *const Self, n: i64,
                            d: i64, out: *mut Self) -> i32;
}

impl GpuFloat for f64 {
    unsafe fn fit_raw(ctx: *mut ffi::fk_ctx, x: *const f64, n: i64, d: i64, p: *const ffi::fk_kmeans_params,
                      init: *const f64, centers: *mut f64, labels: *mut u64, inertia: *mut f64, n_iter: *mut i64,
                      report: *mut ffi::fk_fit_report) -> i32 {
        unsafe { ffi::fk_kmeans_fit_f64(ctx, x, n, d, p, init, centers, labels, inertia, n_iter, report) }
    }
    unsafe fn predict_raw(ctx: *mut ffi::fk_ctx, c: *const f64, k: i64, d_fit: i64, x: *const f64, n: i64, d: i64,
                          labels: *mut u64) -> i32 {
        unsafe { ffi::fk_kmeans_predict_f64(ctx, c, k, d_fit, x, n, d, ffi::FK_PRECISION_PLAIN, labels) }
    }
    unsafe fn transform_raw(ctx: *mut ffi::fk_ctx, c: *const f64, k: i64, d_fit: i64, x: *const f64, n: i64,
                            d: i64, out: *mut f64) -> i32 {
        unsafe { ffi::fk_kmeans_transform_f64(ctx, c, k, d_fit, x, n, d, out) }
    }
}

impl GpuFloat for f32 {
    unsafe fn fit_raw(ctx: *mut ffi::fk_ctx, x: *const f32, n: i64, d: i64, p: *const ffi::fk_kmeans_params,
                      init: *const f32, centers: *mut f32, labels: *mut u64, inertia: *mut f32, n_iter: *mut i64,
                      report: *mut ffi::fk_fit_report) -> i32 {
        unsafe { ffi::fk_kmeans_fit_f32(ctx, x, n, d, p, init, centers, labels, inertia, n_iter, report) }
    }
    unsafe fn predict_raw(ctx: *mut ffi::fk_ctx, c: *const f32, k: i64, d_fit: i64, x: *const f32, n: i64, d: i64,
                          labels: *mut u64) -> i32 {
        unsafe { ffi::fk_kmeans_predict_f32(ctx, c, k, d_fit, x, n, d, ffi::FK_PRECISION_PLAIN, labels) }
    }
    unsafe fn transform_raw(ctx: *mut ffi::fk_ctx, c: *const f32, k: i64, d_fit: i64, x: *const f32, n: i64,
                            d: i64, out: *mut f32) -> i32 {
        unsafe { ffi::fk_kmeans_transform_f32(ctx, c, k, d_fit, x, n, d, out) }
    }
}

fn params(n_clusters: usize, max_iter: usize, tol: f64, n_init: usize, random_state: Option<u64>,
          precision: Precision) -> ffi::fk_kmeans_params {
    let mut p = ffi::fk_kmeans_params {
        n_clusters: 0,
        max_iter: 0,
        tol: 0.0,
        n_init: 0,
        random_state: 0,
        has_random_state: 0,
        precision: 0,
        draws: null(),
        n_draws: 0,
        collect_timing: 0,
        reserved: 0,
    };
    unsafe { ffi::fk_kmeans_params_default(&mut p, n_clusters as i64) };
    p.max_iter = max_iter as i64;
    p.tol = tol;
    p.n_init = n_init as i64;
    if let Some(s) = random_state {
        p.random_state = s;
        p.has_random_state = 1;
    }
    p.precision = precision.code();
    p
}

/// Fit::fit of KMeans<F> (kmeans.rs:403-513) on the GPU: the fitted centres,
/// labels (those of the last assignment of the kept run), inertia and n_iter.
/// A non-C-contiguous `x` is read through its standard layout (the reference
/// reads rows with `as_slice`).
pub fn fit_lloyd<F: GpuFloat>(n_clusters: usize, max_iter: usize, tol: F, n_init: usize, random_state: Option<u64>,
                              x: &Array2<F>) -> Result<(Array2<F>, Array1<usize>, F, usize), FerroError> {
    let x = x.as_standard_layout();
    let (n, d) = x.dim();
    let p = params(n_clusters, max_iter, tol.to_f64().unwrap_or(0.0), n_init, random_state, Precision::Plain);
    let mut centers = Array2::<F>::zeros((n_clusters, d));
    let mut labels = vec![0u64; n];
    let mut inertia = F::zero();
    let mut n_iter = 0i64;
    let shape = Shape { k: n_clusters, n, d_fit: d, d };
    with_ctx(|ctx| {
        let st = unsafe {
            F::fit_raw(ctx, x.as_ptr(), n as i64, d as i64, &p, null(), centers.as_mut_ptr(), labels.as_mut_ptr(),
                       &mut inertia, &mut n_iter, null_mut())
        };
        check(st, &shape, "KMeans requires at least n_clusters samples")
    })?;
    Ok((centers, labels.into_iter().map(|l| l as usize).collect(), inertia, n_iter as usize))
}

/// Predict::predict of FittedKMeans<F> (kmeans.rs:528-553): the nearest
/// centre of each row, lowest index on ties.
pub fn predict_nearest<F: GpuFloat>(centers: &Array2<F>, x: &Array2<F>) -> Result<Array1<usize>, FerroError> {
    let c = centers.as_standard_layout();
    let x = x.as_standard_layout();
    let (k, d_fit) = c.dim();
    let (n, d) = x.dim();
    let mut labels = vec![0u64; n];
    let shape = Shape { k, n, d_fit, d };
    with_ctx(|ctx| {
        let st = unsafe {
            F::predict_raw(ctx, c.as_ptr(), k as i64, d_fit as i64, x.as_ptr(), n as i64, d as i64,
                           labels.as_mut_ptr())
        };
        check(st, &shape, "KMeans::predict")
    })?;
    Ok(labels.into_iter().map(|l| l as usize).collect())
}

/// Transform::transform of FittedKMeans<F> (kmeans.rs:568-617): the
/// Euclidean distance of each row to each centre.
pub fn transform_distances<F: GpuFloat>(centers: &Array2<F>, x: &Array2<F>) -> Result<Array2<F>, FerroError> {
    let c = centers.as_standard_layout();
    let x = x.as_standard_layout();
    let (k, d_fit) = c.dim();
    let (n, d) = x.dim();
    let mut out = Array2::<F>::zeros((n, k));
    let shape = Shape { k, n, d_fit, d };
    with_ctx(|ctx| {
        let st = unsafe {
            F::transform_raw(ctx, c.as_ptr(), k as i64, d_fit as i64, x.as_ptr(), n as i64, d as i64,
                             out.as_mut_ptr())
        };
        check(st, &shape, "KMeans::transform")
    })?;
    Ok(out)
}

/// KMeans configuration (unfitted): the fields, defaults and builders of
/// `ferrolearn_cluster::KMeans<F>` (kmeans.rs:55-113), plus the contraction
/// precision.
#[derive(Debug, Clone)]
pub struct CudaKMeans<F> {
    /// Number of clusters to form.
    pub n_clusters: usize,
    /// Maximum number of Lloyd iterations per run (default 300).
    pub max_iter: usize,
    /// Stop when the largest centre movement is below this (default 1e-4).
    pub tol: F,
    /// Number of runs; the lowest inertia is kept (default 10).
    pub n_init: usize,
    /// Seed of the k-means++ draws (run r: seed + r; None = 0).
    pub random_state: Option<u64>,
    /// Arithmetic of the distance contraction (default Plain).
    pub precision: Precision,
}

impl<F: Float> CudaKMeans<F> {
    /// `KMeans::new(n_clusters)` with the reference's defaults.
    #[must_use]
    pub fn new(n_clusters: usize) -> Self {
        Self {
            n_clusters,
            max_iter: 300,
            tol: F::from(1e-4).unwrap_or_else(F::epsilon),
            n_init: 10,
            random_state: None,
            precision: Precision::Plain,
        }
    }
    #[must_use]
    pub fn with_max_iter(mut self, max_iter: usize) -> Self {
        self.max_iter = max_iter;
        self
    }
    #[must_use]
    pub fn with_tol(mut self, tol: F) -> Self {
        self.tol = tol;
        self
    }
    #[must_use]
    pub fn with_n_init(mut self, n_init: usize) -> Self {
        self.n_init = n_init;
        self
    }
    #[must_use]
    pub fn with_random_state(mut self, seed: u64) -> Self {
        self.random_state = Some(seed);
        self
    }
    /// The tensor-core precisions apply to `CudaKMeans<f64>` fitted on f32 rows.
    #[must_use]
    pub fn with_precision(mut self, precision: Precision) -> Self {
        self.precision = precision;
        self
    }
}

/// Fitted model: the getters of `FittedKMeans<F>` (kmeans.rs:121-156).
#[derive(Debug, Clone)]
pub struct FittedCudaKMeans<F> {
    cluster_centers_: Array2<F>,
    labels_: Array1<usize>,
    inertia_: F,
    n_iter_: usize,
    precision: Precision,
}

impl<F: Float> FittedCudaKMeans<F> {
    /// Cluster centres, shape (n_clusters, n_features).
    #[must_use]
    pub fn cluster_centers(&self) -> &Array2<F> {
        &self.cluster_centers_
    }
    /// Label of each training row.
    #[must_use]
    pub fn labels(&self) -> &Array1<usize> {
        &self.labels_
    }
    /// Sum of squared distances of the training rows to their centres.
    #[must_use]
    pub fn inertia(&self) -> F {
        self.inertia_
    }
    /// Lloyd iterations of the kept run.
    #[must_use]
    pub fn n_iter(&self) -> usize {
        self.n_iter_
    }
}

impl<F: GpuFloat> Fit<Array2<F>, ()> for CudaKMeans<F> {
    type Fitted = FittedCudaKMeans<F>;
    type Error = FerroError;

    fn fit(&self, x: &Array2<F>, _y: &()) -> Result<FittedCudaKMeans<F>, FerroError> {
        if self.precision != Precision::Plain {
            return Err(FerroError::InvalidParameter {
                name: "precision".into(),
                reason: "the tensor-core precisions fit KMeans<f64> on f32 rows (Fit<Array2<f32>, ()> for \
                         CudaKMeans<f64>)"
                    .into(),
            });
        }
        let (c, l, inertia, n_iter) =
            fit_lloyd(self.n_clusters, self.max_iter, self.tol, self.n_init, self.random_state, x)?;
        Ok(FittedCudaKMeans { cluster_centers_: c, labels_: l, inertia_: inertia, n_iter_: n_iter,
                              precision: Precision::Plain })
    }
}

/// KMeans<f64> semantics on rows stored as f32 (each value widened exactly):
/// the entry point of the tensor-core precisions, whose labels equal the
/// FP64 direct form's.
impl Fit<Array2<f32>, ()> for CudaKMeans<f64> {
    type Fitted = FittedCudaKMeans<f64>;
    type Error = FerroError;

    fn fit(&self, x: &Array2<f32>, _y: &()) -> Result<FittedCudaKMeans<f64>, FerroError> {
        let x = x.as_standard_layout();
        let (n, d) = x.dim();
        let p = params(self.n_clusters, self.max_iter, self.tol, self.n_init, self.random_state, self.precision);
        let mut centers = Array2::<f64>::zeros((self.n_clusters, d));
        let mut labels = vec![0u64; n];
        let (mut inertia, mut n_iter) = (0.0f64, 0i64);
        let shape = Shape { k: self.n_clusters, n, d_fit: d, d };
        with_ctx(|ctx| {
            let st = unsafe {
                ffi::fk_kmeans_fit_f32x64(ctx, x.as_ptr(), n as i64, d as i64, &p, null(), centers.as_mut_ptr(),
                                          labels.as_mut_ptr(), &mut inertia, &mut n_iter, null_mut())
            };
            check(st, &shape, "KMeans requires at least n_clusters samples")
        })?;
        Ok(FittedCudaKMeans { cluster_centers_: centers, labels_: labels.into_iter().map(|l| l as usize).collect(),
                              inertia_: inertia, n_iter_: n_iter as usize, precision: self.precision })
    }
}

impl<F: GpuFloat> CudaKMeans<F> {
    /// `fit_predict` (kmeans.rs:522-525): fit, then predict the same rows
    /// with the final centres (which can differ from `labels()`, the
    /// assignment before the last update).
    pub fn fit_predict(&self, x: &Array2<F>) -> Result<Array1<usize>, FerroError> {
        let fitted = self.fit(x, &())?;
        fitted.predict(x)
    }
}

impl<F: GpuFloat> Predict<Array2<F>> for FittedCudaKMeans<F> {
    type Output = Array1<usize>;
    type Error = FerroError;

    fn predict(&self, x: &Array2<F>) -> Result<Array1<usize>, FerroError> {
        predict_nearest(&self.cluster_centers_, x)
    }
}

/// Predict on f32 rows with the model's precision (KMeans<f64> semantics).
impl Predict<Array2<f32>> for FittedCudaKMeans<f64> {
    type Output = Array1<usize>;
    type Error = FerroError;

    fn predict(&self, x: &Array2<f32>) -> Result<Array1<usize>, FerroError> {
        let c = self.cluster_centers_.as_standard_layout();
        let x = x.as_standard_layout();
        let (k, d_fit) = c.dim();
        let (n, d) = x.dim();
        let mut labels = vec![0u64; n];
        let shape = Shape { k, n, d_fit, d };
        with_ctx(|ctx| {
            let st = unsafe {
                ffi::fk_kmeans_predict_f32x64(ctx, c.as_ptr(), k as i64, d_fit as i64, x.as_ptr(), n as i64,
                                              d as i64, self.precision.code(), labels.as_mut_ptr())
            };
            check(st, &shape, "KMeans::predict")
        })?;
        Ok(labels.into_iter().map(|l| l as usize).collect())
    }
}

impl<F: GpuFloat> Transform<Array2<F>> for FittedCudaKMeans<F> {
    type Output = Array2<F>;
    type Error = FerroError;

    fn transform(&self, x: &Array2<F>) -> Result<Array2<F>, FerroError> {
        transform_distances(&self.cluster_centers_, x)
    }
}
