// ba_oracle.cpp -- CPU FP64 restatement of plabundle's online reduced-Schur bundle adjustment.
//
// TEST INFRASTRUCTURE ONLY (see ba_oracle.h).  Parity unpinned: the reference cannot be
// built here, so this is a restatement of its in-tree algorithm; every function cites the
// reference file:line it follows.  It doubles as the timed CPU baseline ("port" kind):
// OpenMP track partitions with per-thread partial sums and an ordered merge, as the
// reference does (src/internal/BundleAdjustPlaMatrixReferenceSchur.cpp:748-927).
#include "ba_oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

constexpr int kP = 13;  // primary block size (BundleAdjustPlaMatrixProblem.h:41)
constexpr int kE = 3;   // eliminated block size (BundleAdjustPlaMatrixProblem.h:42)
constexpr double kInf = std::numeric_limits<double>::infinity();

enum Status { NotRun = 0, Success, NoConvergence, Cancelled, InvalidInput, Unsupported, BackendUnavailable,
              NumericalFailure };

struct Camera {
    double R[9];  // camera-to-world rotation, row-major
    double C[3];  // centre in world
    double fx, fy, cx, cy, k1, k2, k3, p1, p2;
    double su, sv;
    bool flip;
    double width, height;
};

Camera loadCamera(const double* c) {
    Camera cam{};
    std::memcpy(cam.R, c, 9 * sizeof(double));
    std::memcpy(cam.C, c + 9, 3 * sizeof(double));
    cam.fx = c[12]; cam.fy = c[13]; cam.cx = c[14]; cam.cy = c[15];
    cam.k1 = c[16]; cam.k2 = c[17]; cam.k3 = c[18]; cam.p1 = c[19]; cam.p2 = c[20];
    cam.su = c[21] < 0 ? -1.0 : 1.0; cam.sv = c[22] < 0 ? -1.0 : 1.0;
    cam.flip = c[23] != 0.0;
    cam.width = c[24]; cam.height = c[25];
    return cam;
}

void storeCamera(const Camera& cam, double* c) {
    std::fill(c, c + ORC_CAMERA_STRIDE, 0.0);
    std::memcpy(c, cam.R, 9 * sizeof(double));
    std::memcpy(c + 9, cam.C, 3 * sizeof(double));
    c[12] = cam.fx; c[13] = cam.fy; c[14] = cam.cx; c[15] = cam.cy;
    c[16] = cam.k1; c[17] = cam.k2; c[18] = cam.k3; c[19] = cam.p1; c[20] = cam.p2;
    c[21] = cam.su; c[22] = cam.sv; c[23] = cam.flip ? 1.0 : 0.0; c[24] = cam.width; c[25] = cam.height;
}

// CameraState::parameterBlock (CameraState.cpp:164-185); b2, k4, p3, p4 are not part of this
// camera model and stay zero.
std::array<double, kP> parameterBlock(const Camera& c) {
    std::array<double, kP> p{};
    p[0] = c.fx;
    p[1] = (c.fx > 0 && c.fy > 0) ? std::log(c.fy / c.fx) : std::numeric_limits<double>::quiet_NaN();
    p[2] = c.cx; p[3] = c.cy; p[4] = c.k1; p[5] = c.k2; p[6] = c.k3; p[7] = c.p1; p[8] = c.p2;
    return p;
}

// CameraState::supportedParameters (CameraState.cpp:187-204) for a Brown-Conrady frame camera
// with the OpenCV tangential convention and no b2/k4 terms.
std::array<bool, kP> supportedParameters() {
    std::array<bool, kP> m{};
    for (int i = 0; i < 9; ++i) m[i] = true;
    return m;
}

struct Obs {
    int cam;
    double u, v, w, s;
};

// BundleAdjustValidation.cpp:304-326
double sanitizedWeight(const Obs& o) { return std::isfinite(o.w) && o.w > 0.0 ? o.w : 0.0; }
double sanitizedScale(const Obs& o) { return std::isfinite(o.s) && o.s > 0.0 ? o.s : 1.0; }
bool obsDataUsable(const Obs& o) { return std::isfinite(o.u) && std::isfinite(o.v) && sanitizedWeight(o) > 0.0; }
bool obsUsable(const Obs& o, size_t n_cams) {
    return o.cam >= 0 && static_cast<size_t>(o.cam) < n_cams && obsDataUsable(o);
}

// Projection of BundleAdjustProjection.h:58-91 / :121-142.  Returns false for points not in
// front of the camera (forward depth <= 1e-9) or non-finite pixels.
struct ProjectionDerivatives {
    double px[2];
    double xc[3];
    double x, y, r2, radial, xd, yd;
    double dcam[6];  // d pixel / d camera-frame point (2x3)
};

bool projectFull(const Camera& c, const double X[3], ProjectionDerivatives* out, bool derivatives) {
    const double d0 = X[0] - c.C[0], d1 = X[1] - c.C[1], d2 = X[2] - c.C[2];
    const double xc = c.R[0] * d0 + c.R[3] * d1 + c.R[6] * d2;
    const double yc = c.R[1] * d0 + c.R[4] * d1 + c.R[7] * d2;
    const double zc = c.R[2] * d0 + c.R[5] * d1 + c.R[8] * d2;
    const double fwd = c.flip ? -zc : zc;
    if (!(fwd > 1e-9)) return false;
    const double x = xc / zc, y = yc / zc;
    const double r2 = x * x + y * y;
    const double radial = 1.0 + c.k1 * r2 + c.k2 * r2 * r2 + c.k3 * r2 * r2 * r2;
    const double xy2 = 2.0 * x * y;
    const double xd = x * radial + c.p1 * xy2 + c.p2 * (r2 + 2.0 * x * x);
    const double yd = y * radial + c.p1 * (r2 + 2.0 * y * y) + c.p2 * xy2;
    out->px[0] = c.su * c.fx * xd + c.cx;
    out->px[1] = c.sv * c.fy * yd + c.cy;
    out->xc[0] = xc; out->xc[1] = yc; out->xc[2] = zc;
    out->x = x; out->y = y; out->r2 = r2; out->radial = radial; out->xd = xd; out->yd = yd;
    if (!std::isfinite(out->px[0]) || !std::isfinite(out->px[1])) return false;
    if (derivatives) {
        const double dr = c.k1 + 2.0 * c.k2 * r2 + 3.0 * c.k3 * r2 * r2;
        const double dxd_dx = radial + 2.0 * x * x * dr + 2.0 * c.p1 * y + 6.0 * c.p2 * x;
        const double dxd_dy = 2.0 * x * y * dr + 2.0 * c.p1 * x + 2.0 * c.p2 * y;
        const double dyd_dx = 2.0 * x * y * dr + 2.0 * c.p1 * x + 2.0 * c.p2 * y;
        const double dyd_dy = radial + 2.0 * y * y * dr + 6.0 * c.p1 * y + 2.0 * c.p2 * x;
        const double du_dx = c.su * c.fx * dxd_dx, du_dy = c.su * c.fx * dxd_dy;
        const double dv_dx = c.sv * c.fy * dyd_dx, dv_dy = c.sv * c.fy * dyd_dy;
        const double iz = 1.0 / zc;
        out->dcam[0] = du_dx * iz;
        out->dcam[1] = du_dy * iz;
        out->dcam[2] = -(du_dx * x + du_dy * y) * iz;
        out->dcam[3] = dv_dx * iz;
        out->dcam[4] = dv_dy * iz;
        out->dcam[5] = -(dv_dx * x + dv_dy * y) * iz;
    }
    return true;
}

struct RobustEval {
    double cost, weight;
};

// evaluateImageRobustLoss (BundleAdjustPlaMatrixProjection.cpp:75-109).
bool robustLoss(double s, int loss, double scale, RobustEval* out) {
    if (!std::isfinite(s) || s < 0.0) return false;
    if (!std::isfinite(scale) || scale <= 0.0) return false;
    if (loss == 0) { *out = {0.5 * s, 1.0}; return true; }
    const double c2 = scale * scale;
    if (loss == 1) {
        if (s <= c2) { *out = {0.5 * s, 1.0}; return true; }
        const double n = std::sqrt(s);
        *out = {scale * n - 0.5 * c2, scale / n};
        return true;
    }
    if (loss == 2) {
        const double ratio = s / c2;
        *out = {0.5 * c2 * std::log1p(ratio), 1.0 / (1.0 + ratio)};
        return true;
    }
    return false;
}

// referencePointScale (BundleAdjustPlaMatrixAssembly.cpp:31-40).
double referencePointScale(const double* p) {
    const double length = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    const double scaled = length / 1000.0;
    if (!std::isfinite(scaled) || scaled == 0.0) return 1.0;
    return scaled / std::atan(scaled);
}

struct Lin {
    double r[2];
    double Jp[6];       // 2x3 point Jacobian (scaled by the reference point scale)
    double Jc[12];      // 2x6 camera Jacobian [rot(3), centre(3)]
    double Ji[2 * kP];  // 2x13 intrinsic Jacobian
    double nw;
    double cost;
};

// linearizeObservation (BundleAdjustPlaMatrixProjection.cpp:176-285) with the reference point
// parameterisation (:216-262) and linearizeObservationWithActiveIntrinsics (:319-354); the
// intrinsic columns follow CameraState::linearize (CameraState.cpp:427-474).
bool linearize(const Camera& cam, const std::array<bool, kP>& activeInt, const double X[3], const Obs& o, int loss,
               double scale, bool refParam, Lin* L) {
    if (!obsDataUsable(o)) return false;
    ProjectionDerivatives pd;
    if (!projectFull(cam, X, &pd, true)) return false;
    std::memset(L, 0, sizeof(Lin));
    L->r[0] = pd.px[0] - o.u;
    L->r[1] = pd.px[1] - o.v;
    const double* R = cam.R;
    for (int pa = 0; pa < 2; ++pa) {
        for (int wa = 0; wa < 3; ++wa) {
            double d = 0.0;
            for (int ca = 0; ca < 3; ++ca) d += pd.dcam[pa * 3 + ca] * R[wa * 3 + ca];
            L->Jp[pa * 3 + wa] = d;
            L->Jc[pa * 6 + 3 + wa] = -d;
        }
        const double* pj = L->Jp + pa * 3;
        const double dx = X[0] - cam.C[0], dy = X[1] - cam.C[1], dz = X[2] - cam.C[2];
        L->Jc[pa * 6 + 0] = pj[1] * dz - pj[2] * dy;
        L->Jc[pa * 6 + 1] = -pj[0] * dz + pj[2] * dx;
        L->Jc[pa * 6 + 2] = pj[0] * dy - pj[1] * dx;
        if (refParam) {
            const double t[3] = {dx, -dy, -dz};
            const double tc[3][3] = {{0.0, -t[2], t[1]}, {t[2], 0.0, -t[0]}, {-t[1], t[0], 0.0}};
            const double sg[3] = {1.0, -1.0, -1.0};
            for (int k = 0; k < 3; ++k) {
                double d = 0.0;
                for (int ca = 0; ca < 3; ++ca) {
                    double lu = 0.0;
                    for (int ta = 0; ta < 3; ++ta) lu += R[ta * 3 + ca] * sg[ta] * tc[k][ta];
                    d += pd.dcam[pa * 3 + ca] * lu;
                }
                L->Jc[pa * 6 + k] = d;
            }
        }
    }
    if (refParam) {
        const double s = referencePointScale(X);
        for (double& v : L->Jp) v *= s;
    }
    double w = sanitizedWeight(o);
    const double ms = sanitizedScale(o);
    w /= ms * ms;
    RobustEval rb;
    if (!robustLoss(w * (L->r[0] * L->r[0] + L->r[1] * L->r[1]), loss, scale, &rb)) return false;
    L->nw = w * rb.weight;
    L->cost = rb.cost;
    // Intrinsic columns: [fx, log(fy/fx), cx, cy, k1, k2, k3, p1, p2].
    const double aspect = cam.fx > 0 ? cam.fy / cam.fx : 1.0;
    const double x = pd.x, y = pd.y, r2 = pd.r2;
    const double colU[9] = {cam.su * pd.xd, 0.0, 1.0, 0.0, cam.su * cam.fx * x * r2, cam.su * cam.fx * x * r2 * r2,
                            cam.su * cam.fx * x * r2 * r2 * r2, cam.su * cam.fx * 2.0 * x * y,
                            cam.su * cam.fx * (r2 + 2.0 * x * x)};
    const double colV[9] = {cam.sv * pd.yd * aspect, cam.sv * cam.fy * pd.yd, 0.0, 1.0, cam.sv * cam.fy * y * r2,
                            cam.sv * cam.fy * y * r2 * r2, cam.sv * cam.fy * y * r2 * r2 * r2,
                            cam.sv * cam.fy * (r2 + 2.0 * y * y), cam.sv * cam.fy * 2.0 * x * y};
    const auto sup = supportedParameters();
    for (int p = 0; p < 9; ++p) {
        if (activeInt[p] && sup[p]) {
            L->Ji[p] = colU[p];
            L->Ji[kP + p] = colV[p];
        }
    }
    for (double v : L->Ji)
        if (!std::isfinite(v)) return false;
    return std::isfinite(L->nw) && std::isfinite(L->cost);
}

double finiteMedian(std::vector<double> v, double fallback) {
    v.erase(std::remove_if(v.begin(), v.end(), [](double a) { return !std::isfinite(a); }), v.end());
    if (v.empty()) return fallback;
    std::sort(v.begin(), v.end());
    const size_t n = v.size();
    return n % 2 ? v[n / 2] : 0.5 * (v[n / 2 - 1] + v[n / 2]);
}

struct Group {
    std::array<double, kP> params{}, prior{}, invSigma{}, lower{}, upper{};
    std::array<bool, kP> enabled{};
    double focalRef = 1.0, aspectRef = 1.0;
};

struct Active {
    std::vector<char> activeTrack;
    std::vector<int> cameraBlock, intrinsicBlockByCamera, calibGroupByCamera, trackBlock;
    std::vector<int> trackPrimaryBlock;  // scale-bar tracks promoted to primary point blocks, else -1
    // rigs (BundleAdjustPlaMatrixProblem.h:13-39): per camera, the capture / sensor index and block
    std::vector<int> rigCaptureIndexByCamera, rigSensorIndexByCamera, rigCaptureBlockByCamera, rigSensorBlockByCamera;
    int rigCaptureBlockCount = 0, rigSensorBlockCount = 0;
    int primaryBlockCount = 0, cameraBlockCount = 0, intrinsicBlockCount = 0, trackBlockCount = 0;
    int promotedTrackBlockCount = 0;
    int activeTrackCount = 0, observationCount = 0, rejectedInitialTracks = 0;
};

// A rig capture (rig-to-world rotation, rig centre) or sensor (camera-to-rig rotation, camera centre
// in the rig): a rotation R (row-major) and a centre C.
struct RigPose {
    double R[9];
    double C[3];
};

struct State {
    std::vector<Camera> cams;
    std::vector<std::array<double, 3>> points;
    std::vector<Group> groups;
    std::vector<RigPose> captures, sensors;  // rig problems
};

struct OffDiagSlot {
    int row, col;
};

struct BackSub {
    bool valid = false;
    double Vinv[9];
    double rhs[3];
    std::vector<int> blocks;
    std::vector<std::array<double, kP * kE>> cross;
};

struct GeneralEquations;

struct Oracle {
    std::vector<Camera> inputCams, refCams;
    std::vector<std::array<double, 3>> initialPoints;
    std::vector<int64_t> offs;
    std::vector<Obs> obs;
    orc_options opt;
    std::vector<int> fixedCams, fixedTracks;
    std::vector<int> groupIds;
    int gaugeAnchor = -1, gaugeScale = -1;
    double gaugeBaseline = 0.0;
    Active active;
    State state;
    int threads = 1;
    // reduced system
    bool topologyReady = false;
    std::vector<int> lookup;  // P*P
    std::vector<OffDiagSlot> pairs;
    std::vector<double> diag, off, gradient, directRhs;
    std::vector<BackSub> backSub;
    std::vector<std::size_t> boundaries;
    double lastCost = 0.0;
    bool lastSingular = false;

    // control points: per track, the linearisable constraints as J = sqrt(weight) W and target P
    struct ControlPoint {
        double J[9];
        double P[3];
    };
    std::vector<std::vector<ControlPoint>> controlPoints;
    std::vector<std::array<double, 3>> gaugeTargets;  // valid targets of tracks with usable observations
    bool hasControlPoints = false;
    // scale bars: tracks, measured distance and residual scale sqrt(weight) / sigma
    struct ScaleBar {
        int a, b;
        double length, scale, weight;
    };
    std::vector<ScaleBar> scaleBars;

    // block normal equations of the general path (orc_general_build)
    std::shared_ptr<GeneralEquations> general;

    // rig topology: input captures and sensors, (rigId, fixed flag) of each, per-camera binding
    bool hasRig = false;
    std::vector<RigPose> inputCaptures, inputSensors;
    std::vector<int> captureInfo, sensorInfo;
    std::vector<int> cameraCapture, cameraSensor;

    size_t nt() const { return offs.size() - 1; }
    // useReferencePointParameterization (BundleAdjustPlaMatrixAssembly.cpp:24-30)
    bool refParam() const { return !hasControlPoints && scaleBars.empty() && !hasRig; }
};

bool isCameraFixed(const Oracle& o, int cam) {
    return std::find(o.fixedCams.begin(), o.fixedCams.end(), cam) != o.fixedCams.end();
}
bool isTrackFixed(const Oracle& o, int t) { return std::binary_search(o.fixedTracks.begin(), o.fixedTracks.end(), t); }

// Cholesky factor of a 3x3 covariance / information matrix with the checks of
// control_point.cpp:34-85 (finite; symmetric to 1e-10 max(1, running max|a|); pivots L_jj^2
// above 1e-12 max(1, max|a|)).
bool controlPointCholesky(const double* a, double L[3][3]) {
    double mx = 0.0;
    for (int i = 0; i < 9; ++i) {
        const int r = i / 3, c = i % 3;
        const double v = a[r * 3 + c], t = a[c * 3 + r];
        if (!std::isfinite(v) || !std::isfinite(t)) return false;
        mx = std::max({mx, std::fabs(v), std::fabs(t)});
        if (std::fabs(v - t) > 1.0e-10 * std::max(1.0, mx)) return false;
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) L[r][c] = 0.0;
    for (int c = 0; c < 3; ++c) {
        for (int r = c; r < 3; ++r) {
            double v = a[r * 3 + c];
            for (int k = 0; k < c; ++k) v -= L[r][k] * L[c][k];
            if (r == c) {
                if (!(v > 0.0)) return false;
                L[c][c] = std::sqrt(v);
            } else {
                L[r][c] = v / L[c][c];
            }
        }
    }
    const double threshold = std::max(1.0, mx) * 1.0e-12;
    for (int d = 0; d < 3; ++d)
        if (!(L[d][d] * L[d][d] > threshold) || !std::isfinite(L[d][d] * L[d][d])) return false;
    return true;
}

// makeControlPointWhitening (control_point.cpp:91-165) and validateControlPointConstraint
// (:205-220): the whitening W with W^T W the information of the target.  rec: target (3),
// sigma, weight, kind, matrix (9).
bool controlPointWhitening(const double* rec, double W[9]) {
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(rec[a])) return false;
    if (!std::isfinite(rec[4]) || rec[4] <= 0.0) return false;
    const int kind = static_cast<int>(rec[5]);
    const double* m = rec + 6;
    std::fill(W, W + 9, 0.0);
    if (kind == 0) {
        if (!std::isfinite(rec[3]) || rec[3] <= 0.0) return false;
        W[0] = W[4] = W[8] = 1.0 / rec[3];
        return true;
    }
    double L[3][3];
    if (kind == 1) {
        if (!controlPointCholesky(m, L)) return false;
        // W = L^-1 column by column (forward substitution of L w = e_c)
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) {
                double v = r == c ? 1.0 : 0.0;
                for (int k = 0; k < r; ++k) v -= L[r][k] * W[k * 3 + c];
                W[r * 3 + c] = v / L[r][r];
            }
        return true;
    }
    if (kind == 2) {
        for (int i = 0; i < 9; ++i)
            if (!std::isfinite(m[i])) return false;
        double info[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) info[r * 3 + c] = m[r] * m[c] + m[3 + r] * m[3 + c] + m[6 + r] * m[6 + c];
        if (!controlPointCholesky(info, L)) return false;
        std::copy(m, m + 9, W);
        return true;
    }
    return false;
}

// Control points of the problem: Problem validation rejects an invalid constraint
// (problem.cpp:253-260); linearizeControlPoint (BundleAdjustPlaMatrixConstraints.cpp:90-116)
// skips one whose weight controlPointWeight * weight is not positive.  The gauge targets are the
// valid constraints of tracks seen by two distinct cameras (BundleAdjustValidation.cpp:94-106,
// :147-236).
// Scale bars: validateProblem (problem.cpp:342-355) rejects an invalid bar; linearizeScaleBar
// (BundleAdjustPlaMatrixConstraints.cpp:118-153) uses weight = scaleBarWeight * weight and the
// residual scale sqrt(weight) / max(1e-9, sigma).
int loadScaleBars(Oracle& o, const orc_problem* pr) {
    o.scaleBars.clear();
    if (pr->n_scale_bars <= 0) return 0;
    if (!pr->scale_bar_tracks || !pr->scale_bar_data) return InvalidInput;
    if (!std::isfinite(o.opt.scale_bar_weight) || !(o.opt.scale_bar_weight > 0.0) ||
        !std::isfinite(o.opt.scale_bar_huber_delta) || o.opt.scale_bar_huber_delta < 0.0)
        return InvalidInput;
    const int nt = static_cast<int>(o.nt());
    for (int i = 0; i < pr->n_scale_bars; ++i) {
        const int a = pr->scale_bar_tracks[2 * i], b = pr->scale_bar_tracks[2 * i + 1];
        const double* d = pr->scale_bar_data + static_cast<size_t>(i) * 3;
        if (a < 0 || b < 0 || a == b || a >= nt || b >= nt || !std::isfinite(d[0]) || !(d[0] > 0.0) ||
            !std::isfinite(d[1]) || !(d[1] > 0.0) || !std::isfinite(d[2]) || !(d[2] > 0.0))
            return InvalidInput;
        const double w = o.opt.scale_bar_weight * d[2];
        o.scaleBars.push_back({a, b, d[0], std::sqrt(w) / std::max(1e-9, d[1]), w});
    }
    return 0;
}

// linearizeScaleBar with finishRobust's Huber loss: r = s (|Xa - Xb| - L), dr/dXa = s (Xa - Xb) /
// |Xa - Xb| = -dr/dXb; false when the points coincide.
bool scaleBarResidual(const Oracle& o, const Oracle::ScaleBar& sb, const double* Xa, const double* Xb, double* r,
                      double J[3], RobustEval* rb) {
    const double d[3] = {Xa[0] - Xb[0], Xa[1] - Xb[1], Xa[2] - Xb[2]};
    const double dist = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (!(dist > 1e-12)) return false;
    *r = sb.scale * (dist - sb.length);
    for (int a = 0; a < 3; ++a) J[a] = sb.scale * d[a] / dist;
    if (!robustLoss((*r) * (*r), 1, o.opt.scale_bar_huber_delta, rb)) return false;
    return std::isfinite(rb->cost) && std::isfinite(rb->weight);
}

int loadControlPoints(Oracle& o, const orc_problem* pr) {
    o.controlPoints.assign(o.nt(), {});
    o.gaugeTargets.clear();
    o.hasControlPoints = pr->n_control_points > 0;
    if (!o.hasControlPoints) return 0;
    if (!pr->control_point_track || !pr->control_point_data) return InvalidInput;
    const double cw = o.opt.control_point_weight;
    if (!std::isfinite(cw) || cw < 0.0 || !std::isfinite(o.opt.control_point_huber_delta) ||
        o.opt.control_point_huber_delta <= 0.0)
        return InvalidInput;
    for (int i = 0; i < pr->n_control_points; ++i) {
        const int t = pr->control_point_track[i];
        if (t < 0 || t >= static_cast<int>(o.nt())) return InvalidInput;
        const double* rec = pr->control_point_data + static_cast<size_t>(i) * 15;
        double W[9];
        if (!controlPointWhitening(rec, W)) return InvalidInput;
        std::set<int> cams;
        for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k) {
            const Obs& ob = o.obs[k];
            if (ob.cam >= 0 && std::isfinite(ob.u) && std::isfinite(ob.v) && std::isfinite(ob.w) && ob.w > 0.0)
                cams.insert(ob.cam);
        }
        if (cams.size() >= 2) o.gaugeTargets.push_back({rec[0], rec[1], rec[2]});
        const double weight = cw * rec[4];
        if (!(weight > 0.0)) continue;
        Oracle::ControlPoint cp;
        const double sw = std::sqrt(weight);
        for (int k = 0; k < 9; ++k) cp.J[k] = sw * W[k];
        for (int a = 0; a < 3; ++a) cp.P[a] = rec[a];
        o.controlPoints[t].push_back(cp);
    }
    return 0;
}

// linearizeControlPoint + finishRobust (BundleAdjustPlaMatrixConstraints.cpp:17-29, :90-116):
// r = J (X - P), Huber of |r|^2 with the control-point delta.  False when not finite (skipped).
bool controlPointResidual(const Oracle& o, const Oracle::ControlPoint& cp, const double* X, double r[3],
                          RobustEval* rb) {
    const double d[3] = {X[0] - cp.P[0], X[1] - cp.P[1], X[2] - cp.P[2]};
    for (int a = 0; a < 3; ++a) r[a] = cp.J[a * 3] * d[0] + cp.J[a * 3 + 1] * d[1] + cp.J[a * 3 + 2] * d[2];
    if (!robustLoss(r[0] * r[0] + r[1] * r[1] + r[2] * r[2], 1, o.opt.control_point_huber_delta, rb)) return false;
    return std::isfinite(rb->cost) && std::isfinite(rb->weight);
}

// hasCompleteControlPointGauge (BundleAdjustValidation.cpp:181-236): three targets, pairwise
// apart, not collinear.
bool completeControlPointGauge(const Oracle& o) {
    const auto& p = o.gaugeTargets;
    for (size_t i = 0; i < p.size(); ++i)
        for (size_t j = i + 1; j < p.size(); ++j) {
            const double u[3] = {p[j][0] - p[i][0], p[j][1] - p[i][1], p[j][2] - p[i][2]};
            const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
            if (uu <= 1.0e-16) continue;
            for (size_t k = j + 1; k < p.size(); ++k) {
                const double v[3] = {p[k][0] - p[i][0], p[k][1] - p[i][1], p[k][2] - p[i][2]};
                const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
                const double x[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
                if (vv > 1.0e-16 && x[0] * x[0] + x[1] * x[1] + x[2] * x[2] > 1.0e-12 * uu * vv) return true;
            }
        }
    return false;
}

// hasControlPointBaselineToFixedCamera (BundleAdjustValidation.cpp:147-179).
bool controlPointBaseline(const Oracle& o, const std::vector<int>& fixedSet) {
    for (const auto& t : o.gaugeTargets)
        for (int f : fixedSet) {
            const double* c = o.inputCams[f].C;
            if (!std::isfinite(c[0]) || !std::isfinite(c[1]) || !std::isfinite(c[2])) continue;
            const double d2 = (t[0] - c[0]) * (t[0] - c[0]) + (t[1] - c[1]) * (t[1] - c[1]) + (t[2] - c[2]) * (t[2] - c[2]);
            if (d2 > 1.0e-16) return true;
        }
    return false;
}

// Gauge normalisation: validateAndNormalizeBundleAdjustOptions
// (BundleAdjustValidation.cpp:772-893) with control points and no pose priors or scale bars.
int normalizeGauge(Oracle& o) {
    const auto& opt = o.opt;
    std::vector<int> sorted = o.fixedCams;
    std::sort(sorted.begin(), sorted.end());
    for (size_t i = 0; i < sorted.size(); ++i) {
        if (sorted[i] < 0 || sorted[i] >= static_cast<int>(o.inputCams.size())) return InvalidInput;
        if (i > 0 && sorted[i] == sorted[i - 1]) return InvalidInput;
    }
    const bool requested = opt.gauge_anchor_camera >= 0 || opt.gauge_scale_camera >= 0 || opt.gauge_baseline > 0.0;
    const int nc = static_cast<int>(o.inputCams.size());
    if (requested && (opt.gauge_anchor_camera < 0 || opt.gauge_scale_camera < 0 || opt.gauge_anchor_camera >= nc ||
                      opt.gauge_scale_camera >= nc || opt.gauge_anchor_camera == opt.gauge_scale_camera ||
                      !std::isfinite(opt.gauge_baseline) || opt.gauge_baseline <= 0.0))
        return InvalidInput;
    o.gaugeAnchor = opt.gauge_anchor_camera;
    o.gaugeScale = opt.gauge_scale_camera;
    o.gaugeBaseline = opt.gauge_baseline;
    std::sort(o.fixedTracks.begin(), o.fixedTracks.end());
    for (size_t i = 0; i < o.fixedTracks.size(); ++i) {
        if (o.fixedTracks[i] < 0 || o.fixedTracks[i] >= static_cast<int>(o.nt())) return InvalidInput;
        if (i > 0 && o.fixedTracks[i] == o.fixedTracks[i - 1]) return InvalidInput;
    }
    if (!opt.refine_camera_pose || opt.gauge_policy == 2 || o.inputCams.empty()) return 0;
    std::vector<int> fixedSet = sorted;
    const bool absolutePose = completeControlPointGauge(o);
    // hasUsableScaleBar (BundleAdjustValidation.cpp:242-259): every loaded bar is usable
    bool absoluteScale = absolutePose || !o.scaleBars.empty() || controlPointBaseline(o, fixedSet);
    if (opt.gauge_policy == 1)
        return (absolutePose && absoluteScale) || fixedSet.size() >= 2 || (fixedSet.size() == 1 && absoluteScale)
                   ? 0
                   : Unsupported;
    if (absolutePose && absoluteScale) return 0;
    if (fixedSet.empty()) {
        o.fixedCams.push_back(0);
        fixedSet.push_back(0);
        absoluteScale = absoluteScale || controlPointBaseline(o, fixedSet);
    }
    if (!absoluteScale && fixedSet.size() < 2) {
        const int anchor = *std::min_element(fixedSet.begin(), fixedSet.end());
        const double* a = o.inputCams[anchor].C;
        int best = -1;
        double bestD = 1.0e-20;
        for (int i = 0; i < nc; ++i) {
            if (std::find(fixedSet.begin(), fixedSet.end(), i) != fixedSet.end()) continue;
            const double* c = o.inputCams[i].C;
            const double dx = c[0] - a[0], dy = c[1] - a[1], dz = c[2] - a[2];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (std::isfinite(d2) && d2 > bestD) { bestD = d2; best = i; }
        }
        if (best < 0) return Unsupported;
        const double* c = o.inputCams[best].C;
        const double dx = c[0] - a[0], dy = c[1] - a[1], dz = c[2] - a[2];
        o.gaugeAnchor = anchor;
        o.gaugeScale = best;
        o.gaugeBaseline = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    return 0;
}

bool hasSharedIntrinsics(const Oracle& o) { return o.opt.intrinsic_mask != 0; }

// prepareActiveProblem (BundleAdjustPlaMatrixProblem.cpp:29-278) for frame cameras without rigs,
// laser ranges or scale bars.
void prepareActive(Oracle& o) {
    Active& a = o.active;
    const size_t nc = o.inputCams.size(), nt = o.nt();
    a.activeTrack.assign(nt, 0);
    a.cameraBlock.assign(nc, -1);
    a.intrinsicBlockByCamera.assign(nc, -1);
    a.calibGroupByCamera.assign(nc, 0);
    a.trackBlock.assign(nt, -1);
    std::vector<char> camHasResidual(nc, 0);
    for (size_t t = 0; t < nt; ++t) {
        const auto& X = o.initialPoints[t];
        if (!std::isfinite(X[0]) || !std::isfinite(X[1]) || !std::isfinite(X[2])) continue;
        int first = -1;
        bool second = false, positive = true;
        int count = 0;
        double sq = 0.0;
        for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k) {
            const Obs& ob = o.obs[k];
            if (!obsUsable(ob, nc)) continue;
            first = first < 0 ? ob.cam : first;
            second = second || ob.cam != first;
            ProjectionDerivatives pd;
            if (!projectFull(o.inputCams[ob.cam], X.data(), &pd, false)) {
                positive = false;
                break;
            }
            const double du = pd.px[0] - ob.u, dv = pd.px[1] - ob.v;
            sq += sanitizedWeight(ob) * (du * du + dv * dv);
            ++count;
        }
        const double rms = count > 0 ? std::sqrt(sq / (2.0 * count)) : kInf;
        if (count < 2 || !second || !positive) continue;
        if (o.opt.max_initial_track_rms > 0.0 && rms > o.opt.max_initial_track_rms) {
            ++a.rejectedInitialTracks;
            continue;
        }
        a.activeTrack[t] = 1;
        ++a.activeTrackCount;
        a.observationCount += count;
        for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k)
            if (obsUsable(o.obs[k], nc)) camHasResidual[o.obs[k].cam] = 1;
    }
    a.rigCaptureIndexByCamera.assign(nc, -1);
    a.rigSensorIndexByCamera.assign(nc, -1);
    a.rigCaptureBlockByCamera.assign(nc, -1);
    a.rigSensorBlockByCamera.assign(nc, -1);
    if (o.hasRig) {
        a.rigCaptureIndexByCamera = o.cameraCapture;
        a.rigSensorIndexByCamera = o.cameraSensor;
    }
    if (o.opt.refine_camera_pose && !o.hasRig) {
        for (size_t c = 0; c < nc; ++c)
            if (camHasResidual[c] && !isCameraFixed(o, static_cast<int>(c))) a.cameraBlock[c] = a.cameraBlockCount++;
    } else if (o.opt.refine_camera_pose) {
        // BundleAdjustPlaMatrixProblem.cpp:156-199
        const size_t ncap = o.inputCaptures.size(), nsen = o.inputSensors.size();
        std::vector<int> captureBlocks(ncap, -1), sensorBlocks(nsen, -1);
        for (size_t k = 0; k < ncap; ++k) {
            bool hasResidual = false;
            bool fixed = o.captureInfo[2 * k + 1] != 0;
            for (size_t c = 0; c < nc; ++c)
                if (a.rigCaptureIndexByCamera[c] == static_cast<int>(k)) {
                    hasResidual = hasResidual || camHasResidual[c];
                    fixed = fixed || isCameraFixed(o, static_cast<int>(c)) || o.gaugeScale == static_cast<int>(c);
                }
            if (hasResidual && !fixed) captureBlocks[k] = a.rigCaptureBlockCount++;
        }
        for (size_t sI = 0; sI < nsen; ++sI) {
            bool hasResidual = false;
            for (size_t c = 0; c < nc; ++c)
                hasResidual = hasResidual || (a.rigSensorIndexByCamera[c] == static_cast<int>(sI) && camHasResidual[c]);
            if (hasResidual && !o.sensorInfo[2 * sI + 1])
                sensorBlocks[sI] = a.rigCaptureBlockCount + a.rigSensorBlockCount++;
        }
        for (size_t c = 0; c < nc; ++c) {
            a.rigCaptureBlockByCamera[c] = captureBlocks[static_cast<size_t>(a.rigCaptureIndexByCamera[c])];
            a.rigSensorBlockByCamera[c] = sensorBlocks[static_cast<size_t>(a.rigSensorIndexByCamera[c])];
        }
        a.cameraBlockCount = a.rigCaptureBlockCount + a.rigSensorBlockCount;
    }
    a.primaryBlockCount = a.cameraBlockCount;
    if (hasSharedIntrinsics(o)) {
        if (!o.groupIds.empty()) a.calibGroupByCamera = o.groupIds;
        std::vector<int> ids;
        for (size_t c = 0; c < nc; ++c) {
            const int id = a.calibGroupByCamera[c];
            auto it = std::find(ids.begin(), ids.end(), id);
            int gi;
            if (it == ids.end()) { gi = static_cast<int>(ids.size()); ids.push_back(id); }
            else gi = static_cast<int>(it - ids.begin());
            a.calibGroupByCamera[c] = gi;
        }
        a.intrinsicBlockCount = static_cast<int>(ids.size());
        for (size_t c = 0; c < nc; ++c) a.intrinsicBlockByCamera[c] = a.primaryBlockCount + a.calibGroupByCamera[c];
        a.primaryBlockCount += a.intrinsicBlockCount;
    }
    // scale-bar tracks become primary point blocks (BundleAdjustPlaMatrixProblem.cpp:235-266)
    std::vector<char> promote(nt, 0);
    for (const auto& sb : o.scaleBars)
        for (int t : {sb.a, sb.b})
            if (a.activeTrack[t] && !isTrackFixed(o, t)) promote[t] = 1;
    a.trackPrimaryBlock.assign(nt, -1);
    a.promotedTrackBlockCount = 0;
    for (size_t t = 0; t < nt; ++t) {
        if (!a.activeTrack[t] || isTrackFixed(o, static_cast<int>(t))) continue;
        if (promote[t]) {
            a.trackPrimaryBlock[t] = a.primaryBlockCount++;
            ++a.promotedTrackBlockCount;
        } else {
            a.trackBlock[t] = a.trackBlockCount++;
        }
    }
}

// initializeIntrinsicGroups (BundleAdjustPlaMatrixModel.cpp:84-231) without the calibration
// transition prior.
void initGroups(Oracle& o) {
    const Active& a = o.active;
    o.state.groups.assign(static_cast<size_t>(a.intrinsicBlockCount), Group{});
    if (o.state.groups.empty()) return;
    const auto& refs = o.refCams.empty() ? o.inputCams : o.refCams;
    struct Samples {
        std::array<std::vector<double>, kP> initial, reference;
        std::array<bool, kP> supported;
    };
    std::vector<Samples> samples(o.state.groups.size());
    for (auto& s : samples) s.supported.fill(true);
    for (size_t c = 0; c < o.inputCams.size(); ++c) {
        auto& s = samples[static_cast<size_t>(a.calibGroupByCamera[c])];
        const auto p = parameterBlock(o.inputCams[c]);
        const auto rp = parameterBlock(refs[c]);
        const auto sup = supportedParameters();
        s.initial[0].push_back(p[0]);
        s.reference[0].push_back(rp[0]);
        s.initial[1].push_back(std::exp(p[1]));
        s.reference[1].push_back(std::exp(rp[1]));
        s.initial[2].push_back(o.inputCams[c].cx - refs[c].cx);
        s.initial[3].push_back(o.inputCams[c].cy - refs[c].cy);
        s.reference[2].push_back(0.0);
        s.reference[3].push_back(0.0);
        for (int i = 4; i < kP; ++i) {
            s.initial[i].push_back(p[i]);
            s.reference[i].push_back(rp[i]);
        }
        for (int i = 0; i < kP; ++i) s.supported[i] = s.supported[i] && sup[i];
    }
    const double* cal = o.opt.calibration;
    const double lowScale = std::max(1.0, cal[26]);
    for (size_t g = 0; g < o.state.groups.size(); ++g) {
        Group& gr = o.state.groups[g];
        gr.lower.fill(-kInf);
        gr.upper.fill(kInf);
        for (int p = 0; p < kP; ++p) gr.enabled[p] = ((o.opt.intrinsic_mask >> p) & 1u) && samples[g].supported[p];
        gr.focalRef = finiteMedian(samples[g].reference[0], 1.0);
        gr.aspectRef = finiteMedian(samples[g].reference[1], 1.0);
        gr.params[0] = std::max(1e-12, finiteMedian(samples[g].initial[0], gr.focalRef));
        gr.params[1] = std::log(std::max(1e-12, finiteMedian(samples[g].initial[1], gr.aspectRef)));
        gr.prior[0] = gr.focalRef;
        gr.prior[1] = std::log(gr.aspectRef);
        for (int p = 2; p < kP; ++p) {
            gr.prior[p] = finiteMedian(samples[g].reference[p], 0.0);
            gr.params[p] = finiteMedian(samples[g].initial[p], gr.prior[p]);
        }
        gr.lower[0] = gr.focalRef * cal[0];
        gr.upper[0] = gr.focalRef * cal[1];
        gr.lower[1] = std::log(gr.aspectRef * cal[2]);
        gr.upper[1] = std::log(gr.aspectRef * cal[3]);
        const double ppLimit = gr.focalRef * cal[4];
        gr.lower[2] = gr.lower[3] = -ppLimit;
        gr.upper[2] = gr.upper[3] = ppLimit;
        const double lim[9] = {cal[8] * lowScale, cal[9], cal[10], cal[11] * lowScale, cal[12] * lowScale,
                               gr.focalRef * cal[13], cal[14], cal[15], cal[16]};
        for (int i = 0; i < 9; ++i) {
            gr.lower[i + 4] = -lim[i];
            gr.upper[i + 4] = lim[i];
        }
        const double ppSigma = std::max(1e-6, gr.focalRef * cal[6]);
        const double sigma[kP] = {cal[5] * gr.focalRef, cal[7], ppSigma, ppSigma, cal[17] * lowScale, cal[18], cal[19],
                                  cal[20] * lowScale, cal[21] * lowScale, gr.focalRef * cal[22], cal[23], cal[24],
                                  cal[25]};
        for (int p = 0; p < kP; ++p) {
            gr.params[p] = std::clamp(gr.params[p], gr.lower[p], gr.upper[p]);
            gr.invSigma[p] = gr.enabled[p] ? 1.0 / std::max(1e-9, sigma[p]) : 0.0;
        }
    }
}

// makeCameraWithSharedIntrinsics (BundleAdjustPlaMatrixProjection.cpp:134-171).
Camera effectiveCamera(const Oracle& o, const State& s, size_t c) {
    Camera e = s.cams[c];
    if (s.groups.empty()) return e;
    const auto& refs = o.refCams.empty() ? o.inputCams : o.refCams;
    const Group& g = s.groups[static_cast<size_t>(o.active.calibGroupByCamera[c])];
    const Camera& src = s.cams[c];
    const double fx = g.enabled[0] ? g.params[0] : src.fx;
    const double srcAspect = src.fx > 1e-12 ? src.fy / src.fx : 1.0;
    const double aspect = g.enabled[1] ? std::exp(g.params[1]) : srcAspect;
    e.fx = fx;
    e.fy = fx * aspect;
    e.cx = g.enabled[2] ? refs[c].cx + g.params[2] : src.cx;
    e.cy = g.enabled[3] ? refs[c].cy + g.params[3] : src.cy;
    double* dist[5] = {&e.k1, &e.k2, &e.k3, &e.p1, &e.p2};
    for (int p = 4; p < 9; ++p)
        if (g.enabled[p]) *dist[p - 4] = g.params[p];
    return e;
}

std::array<bool, kP> activeIntrinsics(const Oracle& o, size_t c) {
    std::array<bool, kP> m{};
    if (o.state.groups.empty()) return m;
    return o.state.groups[static_cast<size_t>(o.active.calibGroupByCamera[c])].enabled;
}

bool usesGaugeTangent(const Oracle& o, size_t c) {
    const int nc = static_cast<int>(o.inputCams.size());
    // a rig camera never takes the tangent (constrained_center, BundleAdjustPlaMatrixAssembly.cpp:204)
    return !o.hasRig && o.gaugeAnchor >= 0 && o.gaugeScale >= 0 && o.gaugeAnchor < nc && o.gaugeScale < nc &&
           c == static_cast<size_t>(o.gaugeScale) && std::isfinite(o.gaugeBaseline) && o.gaugeBaseline > 0.0;
}

std::array<double, 3> targetCoords(const double* v) { return {v[0], -v[1], -v[2]}; }
std::array<double, 3> cross3(const std::array<double, 3>& a, const std::array<double, 3>& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
double norm3(const std::array<double, 3>& a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// referenceGaugeTargetTangentBasis (BundleAdjustPlaMatrixAssembly.cpp:69-99).
std::array<std::array<double, 3>, 2> gaugeBasis(const Oracle& o, const State& s) {
    const auto origin = targetCoords(s.cams[o.gaugeAnchor].C);
    const auto centre = targetCoords(s.cams[o.gaugeScale].C);
    std::array<double, 3> unit{centre[0] - origin[0], centre[1] - origin[1], centre[2] - origin[2]};
    const double len = norm3(unit);
    const double il = len >= 1e-20 ? 1.0 / len : 0.0;
    for (double& v : unit) v *= il;
    int axis = std::abs(unit[0]) > std::abs(unit[1]) ? 1 : 0;
    if (std::abs(unit[axis]) > std::abs(unit[2])) axis = 2;
    std::array<double, 3> ax{};
    ax[axis] = 1.0;
    auto second = cross3(ax, unit);
    const double sl = norm3(second);
    const double isl = sl >= 1e-20 ? 1.0 / sl : 0.0;
    for (double& v : second) v *= isl;
    return {cross3(unit, second), second};
}

// cameraPosePrimaryTerms + observationPrimaryTerms (BundleAdjustPlaMatrixAssembly.cpp:186-342).
// A rig camera's Jacobian is chained to its capture block (rotation column a: J_rot[a] +
// J_ctr (e_a x L) with the lever L = R_rig c_sensor; centre columns J_ctr) and its sensor block
// (columns J_rot R_rig[:, a] and J_ctr R_rig[:, a]) (:207-284); its intrinsic block follows.
struct Terms {
    int blocks[3];
    double J[3][2 * kP];
    int count = 0;
};

Terms primaryTerms(const Oracle& o, const State& s, size_t c, const Lin& L) {
    Terms t;
    std::memset(t.J, 0, sizeof(t.J));
    if (o.hasRig) {
        const int ki = o.active.rigCaptureIndexByCamera[c], si = o.active.rigSensorIndexByCamera[c];
        if (ki >= 0 && si >= 0) {
            const RigPose& cap = s.captures[static_cast<size_t>(ki)];
            const RigPose& sen = s.sensors[static_cast<size_t>(si)];
            double lever[3] = {0, 0, 0};
            for (int w = 0; w < 3; ++w)
                for (int r = 0; r < 3; ++r) lever[w] += cap.R[w * 3 + r] * sen.C[r];
            const int kb = o.active.rigCaptureBlockByCamera[c], sb = o.active.rigSensorBlockByCamera[c];
            if (kb >= 0) {
                double* J = t.J[t.count];
                for (int row = 0; row < 2; ++row) {
                    const double* cr = L.Jc + row * 6;
                    for (int ax = 0; ax < 3; ++ax) {
                        double cd[3] = {0, 0, 0};
                        cd[(ax + 1) % 3] = -lever[(ax + 2) % 3];
                        cd[(ax + 2) % 3] = lever[(ax + 1) % 3];
                        J[row * kP + ax] = cr[ax];
                        for (int w = 0; w < 3; ++w) J[row * kP + ax] += cr[3 + w] * cd[w];
                        J[row * kP + 3 + ax] = cr[3 + ax];
                    }
                }
                t.blocks[t.count++] = kb;
            }
            if (sb >= 0) {
                double* J = t.J[t.count];
                for (int row = 0; row < 2; ++row) {
                    const double* cr = L.Jc + row * 6;
                    for (int ax = 0; ax < 3; ++ax)
                        for (int w = 0; w < 3; ++w) {
                            const double basis = cap.R[w * 3 + ax];
                            J[row * kP + ax] += cr[w] * basis;
                            J[row * kP + 3 + ax] += cr[3 + w] * basis;
                        }
                }
                t.blocks[t.count++] = sb;
            }
        }
        const int ib = o.active.intrinsicBlockByCamera[c];
        if (ib >= 0) {
            std::memcpy(t.J[t.count], L.Ji, sizeof(L.Ji));
            t.blocks[t.count++] = ib;
        }
        return t;
    }
    const int cb = o.active.cameraBlock[c];
    if (cb >= 0) {
        const bool tangent = usesGaugeTangent(o, c);
        std::array<std::array<double, 3>, 2> basis{};
        if (tangent) basis = gaugeBasis(o, s);
        for (int row = 0; row < 2; ++row) {
            const double* src = L.Jc + row * 6;
            for (int k = 0; k < 3; ++k) t.J[0][row * kP + k] = src[k];
            if (tangent) {
                for (int p = 0; p < 2; ++p) {
                    const auto wb = targetCoords(basis[p].data());
                    for (int ax = 0; ax < 3; ++ax) t.J[0][row * kP + 3 + p] += src[3 + ax] * wb[ax];
                }
            } else {
                for (int k = 0; k < 3; ++k) t.J[0][row * kP + 3 + k] = src[3 + k];
            }
        }
        t.blocks[0] = cb;
        t.count = 1;
    }
    const int ib = o.active.intrinsicBlockByCamera[c];
    if (ib >= 0) {
        std::memcpy(t.J[t.count], L.Ji, sizeof(L.Ji));
        t.blocks[t.count] = ib;
        ++t.count;
    }
    return t;
}

// prepareOffDiagonalTopology (BundleAdjustPlaMatrixReferenceSchur.cpp:568-659).
void prepareTopology(Oracle& o) {
    if (o.topologyReady) return;
    const int P = o.active.primaryBlockCount;
    const size_t lsz = static_cast<size_t>(P) * P;
    o.lookup.assign(lsz, -1);
    std::vector<char> connected(lsz, 0);
    auto connect = [&](int l, int r) {
        if (l < 0 || r < 0 || l == r) return;
        connected[static_cast<size_t>(std::min(l, r)) * P + std::max(l, r)] = 1;
    };
    std::vector<int> tb;
    for (size_t t = 0; t < o.nt(); ++t) {
        if (!o.active.activeTrack[t]) continue;
        tb.clear();
        for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k) {
            const Obs& ob = o.obs[k];
            if (!obsUsable(ob, o.inputCams.size())) continue;
            const int b[4] = {o.active.cameraBlock[ob.cam], o.active.rigCaptureBlockByCamera[ob.cam],
                              o.active.rigSensorBlockByCamera[ob.cam], o.active.intrinsicBlockByCamera[ob.cam]};
            for (int l = 0; l < 4; ++l)
                for (int r = l + 1; r < 4; ++r) connect(b[l], b[r]);
            if (o.active.trackBlock[t] >= 0)
                for (int v : b)
                    if (v >= 0) tb.push_back(v);
        }
        if (o.active.trackBlock[t] < 0) continue;
        std::sort(tb.begin(), tb.end());
        tb.erase(std::unique(tb.begin(), tb.end()), tb.end());
        for (size_t l = 0; l < tb.size(); ++l)
            for (size_t r = l + 1; r < tb.size(); ++r) connect(tb[l], tb[r]);
    }
    for (int r = 0; r < P; ++r)
        for (int c = r + 1; c < P; ++c) {
            const size_t li = static_cast<size_t>(r) * P + c;
            if (!connected[li]) continue;
            o.lookup[li] = static_cast<int>(o.pairs.size());
            o.pairs.push_back({r, c});
        }
    o.topologyReady = true;
}

// updateTrackBoundaries (BundleAdjustPlaMatrixReferenceSchur.cpp:538-566).
void trackBoundaries(Oracle& o, int threads) {
    std::vector<size_t> prefix(o.nt() + 1, 0);
    for (size_t t = 0; t < o.nt(); ++t) {
        const size_t w = o.active.activeTrack[t] ? std::max<size_t>(1, static_cast<size_t>(o.offs[t + 1] - o.offs[t]))
                                                 : 1;
        prefix[t + 1] = prefix[t] + w;
    }
    o.boundaries.assign(static_cast<size_t>(threads + 1), o.nt());
    o.boundaries[0] = 0;
    for (int th = 1; th < threads; ++th) {
        const size_t target = prefix.back() * static_cast<size_t>(th) / static_cast<size_t>(threads);
        o.boundaries[th] = static_cast<size_t>(std::lower_bound(prefix.begin(), prefix.end(), target) - prefix.begin());
    }
}

// tryInverse3x3RowMajor restatement: adjugate / determinant, singular when |det| <= tol.
bool inverse3x3(const double* m, double* inv, double tol) {
    const double c00 = m[4] * m[8] - m[5] * m[7];
    const double c01 = m[5] * m[6] - m[3] * m[8];
    const double c02 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    if (!std::isfinite(det) || std::abs(det) <= tol) return false;
    const double id = 1.0 / det;
    inv[0] = c00 * id;
    inv[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    inv[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    inv[3] = c01 * id;
    inv[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    inv[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    inv[6] = c02 * id;
    inv[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    inv[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(inv[i])) return false;
    return true;
}

struct InvalidProjection : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct PointWork {
    double V[9];
    double rhs[3];
    std::vector<int> blocks;
    std::vector<std::array<double, kP * kE>> cross;
    void clear() {
        std::fill(V, V + 9, 0.0);
        std::fill(rhs, rhs + 3, 0.0);
        blocks.clear();
        cross.clear();
    }
    std::array<double, kP * kE>& crossBlock(int b) {
        for (size_t i = 0; i < blocks.size(); ++i)
            if (blocks[i] == b) return cross[i];
        blocks.push_back(b);
        cross.emplace_back();
        cross.back().fill(0.0);
        return cross.back();
    }
};

struct Accumulator {
    double* diag;
    double* directRhs;
    double* schurRhs;
    double* off;
    bool atomic;
    const Oracle* o;
    void add(int rb, int cb, int row, int col, double v) {
        if (rb == cb) {
            diag[static_cast<size_t>(rb) * kP * kP + row * kP + col] += v;
            return;
        }
        const bool ordered = rb < cb;
        const int sr = ordered ? rb : cb, sc = ordered ? cb : rb;
        const int slot = o->lookup[static_cast<size_t>(sr) * o->active.primaryBlockCount + sc];
        if (slot < 0) throw std::logic_error("missing off-diagonal block");
        double& e = off[static_cast<size_t>(slot) * kP * kP + (ordered ? row * kP + col : col * kP + row)];
        if (atomic) {
#pragma omp atomic
            e += v;
        } else {
            e += v;
        }
    }
};

// accumulateObservationPrimaryTerms (BundleAdjustPlaMatrixReferenceSchur.cpp:140-193).
void accumulateDirect(const Terms& t, const Lin& L, Accumulator& acc) {
    int act[3][kP];
    int na[3] = {0, 0, 0};
    for (int k = 0; k < t.count; ++k) {
        for (int p = 0; p < kP; ++p) {
            const double jx = t.J[k][p], jy = t.J[k][kP + p];
            if (jx == 0.0 && jy == 0.0) continue;
            act[k][na[k]++] = p;
            double g = 0.0;
            for (int row = 0; row < 2; ++row) g += L.nw * t.J[k][row * kP + p] * L.r[row];
            acc.directRhs[static_cast<size_t>(t.blocks[k]) * kP + p] -= g;
        }
    }
    for (int l = 0; l < t.count; ++l)
        for (int r = l; r < t.count; ++r)
            for (int li = 0; li < na[l]; ++li) {
                const int row = act[l][li];
                const double lx = t.J[l][row], ly = t.J[l][kP + row];
                for (int ri = 0; ri < na[r]; ++ri) {
                    const int col = act[r][ri];
                    acc.add(t.blocks[l], t.blocks[r], row, col, L.nw * (lx * t.J[r][col] + ly * t.J[r][kP + col]));
                }
            }
}

// accumulatePointTerms (BundleAdjustPlaMatrixReferenceSchur.cpp:195-239).
void accumulatePoint(const Terms& t, const Lin& L, PointWork& pw) {
    for (int c = 0; c < kE; ++c)
        for (int row = 0; row < 2; ++row) {
            const double pv = L.Jp[row * kE + c];
            pw.rhs[c] -= L.nw * pv * L.r[row];
            for (int oth = 0; oth < kE; ++oth) pw.V[c * kE + oth] += L.nw * pv * L.Jp[row * kE + oth];
        }
    for (int k = 0; k < t.count; ++k) {
        auto& cr = pw.crossBlock(t.blocks[k]);
        for (int p = 0; p < kP; ++p) {
            const double jx = t.J[k][p], jy = t.J[k][kP + p];
            if (jx == 0.0 && jy == 0.0) continue;
            for (int e = 0; e < kE; ++e) cr[p * kE + e] += L.nw * (jx * L.Jp[e] + jy * L.Jp[kE + e]);
        }
    }
}

// eliminatePoint (BundleAdjustPlaMatrixReferenceSchur.cpp:350-490).
bool eliminatePoint(double damping, PointWork& pw, Accumulator& acc, BackSub* bs) {
    double dh[9];
    std::memcpy(dh, pw.V, sizeof(dh));
    for (int d = 0; d < kE; ++d) dh[d * kE + d] *= 1.0 + damping;
    double inv[9];
    if (!inverse3x3(dh, inv, 1.0e-15)) {
        bs->valid = false;
        return false;
    }
    const size_t nb = pw.blocks.size();
    std::vector<std::array<double, kP * kE>> red(nb);
    std::vector<std::array<char, kP>> activeRows(nb);
    for (size_t b = 0; b < nb; ++b) {
        red[b].fill(0.0);
        activeRows[b].fill(0);
        for (int row = 0; row < kP; ++row) {
            const double* cr = pw.cross[b].data() + row * kE;
            activeRows[b][row] = cr[0] != 0.0 || cr[1] != 0.0 || cr[2] != 0.0;
            if (!activeRows[b][row]) continue;
            for (int c = 0; c < kE; ++c)
                for (int in = 0; in < kE; ++in) red[b][row * kE + c] += cr[in] * inv[in * kE + c];
        }
        for (int row = 0; row < kP; ++row) {
            if (!activeRows[b][row]) continue;
            double g = 0.0;
            for (int c = 0; c < kE; ++c) g += red[b][row * kE + c] * pw.rhs[c];
            acc.schurRhs[static_cast<size_t>(pw.blocks[b]) * kP + row] -= g;
        }
    }
    for (size_t l = 0; l < nb; ++l)
        for (size_t r = l; r < nb; ++r)
            for (int row = 0; row < kP; ++row) {
                if (!activeRows[l][row]) continue;
                for (int col = 0; col < kP; ++col) {
                    if (!activeRows[r][col]) continue;
                    double h = 0.0;
                    for (int in = 0; in < kE; ++in) h -= red[l][row * kE + in] * pw.cross[r][col * kE + in];
                    acc.add(pw.blocks[l], pw.blocks[r], row, col, h);
                }
            }
    std::memcpy(bs->Vinv, inv, sizeof(inv));
    std::memcpy(bs->rhs, pw.rhs, sizeof(pw.rhs));
    bs->blocks = pw.blocks;
    bs->cross = pw.cross;
    bs->valid = true;
    return true;
}

// Intrinsic priors: assembleReferencePriors (BundleAdjustPlaMatrixReferenceSchur.cpp:492-536);
// addPrimaryResidualBlock adds J^T J to the diagonal block and J^T r to the gradient.
double assemblePriors(Oracle& o) {
    double cost = 0.0;
    for (size_t g = 0; g < o.state.groups.size(); ++g) {
        const Group& gr = o.state.groups[g];
        const int block = o.active.cameraBlockCount + static_cast<int>(g);
        for (int p = 0; p < kP; ++p) {
            if (!gr.enabled[p]) continue;
            const double w = gr.invSigma[p];
            const double r = w * (gr.params[p] - gr.prior[p]);
            cost += 0.5 * r * r;
            o.diag[static_cast<size_t>(block) * kP * kP + p * kP + p] += w * w;
            o.gradient[static_cast<size_t>(block) * kP + p] += w * r;
            o.directRhs[static_cast<size_t>(block) * kP + p] -= w * r;
        }
    }
    return cost;
}

double priorCost(const Oracle& o, const State& s) {
    double cost = 0.0;
    for (const Group& gr : s.groups)
        for (int p = 0; p < kP; ++p) {
            if (!gr.enabled[p]) continue;
            const double r = gr.invSigma[p] * (gr.params[p] - gr.prior[p]);
            cost += 0.5 * r * r;
        }
    (void)o;
    return cost;
}

// buildReferenceReducedNormalEquations (BundleAdjustPlaMatrixReferenceSchur.cpp:675-980).
void build(Oracle& o, double damping, double* costOut, bool* singularOut) {
    if (!std::isfinite(damping) || damping < 0.0) throw std::invalid_argument("invalid damping");
    const int T = std::max(1, std::min<int>(o.threads, static_cast<int>(o.nt())));
    trackBoundaries(o, T);
    prepareTopology(o);
    const int P = o.active.primaryBlockCount;
    const size_t pdim = static_cast<size_t>(P) * kP, ddim = static_cast<size_t>(P) * kP * kP;
    const size_t odim = o.pairs.size() * kP * kP;
    std::vector<std::vector<double>> pDiag(T, std::vector<double>(ddim, 0.0)), pDirect(T, std::vector<double>(pdim, 0.0)),
        pSchur(T, std::vector<double>(pdim, 0.0));
    const size_t slotBudget = 128ull * 1024ull * 1024ull;
    const size_t bytesPerSlot = odim * sizeof(double);
    const size_t within = bytesPerSlot == 0 ? static_cast<size_t>(T) : std::max<size_t>(1, slotBudget / bytesPerSlot);
    const int nSlots = within >= static_cast<size_t>(T) ? T : static_cast<int>(within);
    const bool own = nSlots == T;
    std::vector<std::vector<double>> slots(nSlots, std::vector<double>(odim, 0.0));
    std::vector<double> pCost(T, 0.0);
    std::vector<char> pSingular(T, 0);
    std::vector<std::string> errors(T);
    o.backSub.assign(o.nt(), BackSub{});
    const bool ref = o.refParam();
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int th = 0; th < T; ++th) {
        try {
            Accumulator acc{pDiag[th].data(), pDirect[th].data(), pSchur[th].data(), slots[th % nSlots].data(), !own, &o};
            PointWork pw;
            double cost = 0.0;
            for (size_t t = o.boundaries[th]; t < o.boundaries[th + 1]; ++t) {
                if (!o.active.activeTrack[t]) continue;
                pw.clear();
                const bool elim = o.active.trackBlock[t] >= 0;
                for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k) {
                    const Obs& ob = o.obs[k];
                    if (!obsUsable(ob, o.state.cams.size())) continue;
                    const Camera cam = effectiveCamera(o, o.state, ob.cam);
                    Lin L;
                    if (!linearize(cam, activeIntrinsics(o, ob.cam), o.state.points[t].data(), ob, o.opt.robust_loss,
                                   o.opt.robust_loss_scale, ref, &L))
                        throw InvalidProjection("online Schur linearisation produced an invalid projection");
                    cost += L.cost;
                    const Terms tm = primaryTerms(o, o.state, ob.cam, L);
                    accumulateDirect(tm, L, acc);
                    if (elim) accumulatePoint(tm, L, pw);
                }
                // control points (linearizeTrack, BundleAdjustPlaMatrixReferenceSchur.cpp:331-346) and
                // accumulatePointOnlyConstraint (:241-260)
                for (const auto& cp : o.controlPoints[t]) {
                    double r[3];
                    RobustEval rb;
                    if (!controlPointResidual(o, cp, o.state.points[t].data(), r, &rb)) continue;
                    cost += rb.cost;
                    if (!elim) continue;
                    for (int c = 0; c < kE; ++c)
                        for (int row = 0; row < 3; ++row) {
                            const double jv = cp.J[row * 3 + c];
                            pw.rhs[c] -= rb.weight * jv * r[row];
                            for (int oth = 0; oth < kE; ++oth) pw.V[c * kE + oth] += rb.weight * jv * cp.J[row * 3 + oth];
                        }
                }
                if (elim && !eliminatePoint(damping, pw, acc, &o.backSub[t])) pSingular[th] = 1;
            }
            pCost[th] = cost;
        } catch (const std::exception& e) {
            errors[th] = e.what();
            if (errors[th].empty()) errors[th] = "error";
        }
    }
    o.diag.assign(ddim, 0.0);
    o.off.assign(odim, 0.0);
    o.gradient.assign(pdim, 0.0);
    o.directRhs.assign(pdim, 0.0);
    double cost = 0.0;
    bool singular = false;
    for (int th = 0; th < T; ++th) {
        if (!errors[th].empty()) throw InvalidProjection(errors[th]);
        for (size_t i = 0; i < pdim; ++i) o.directRhs[i] += pDirect[th][i];
        cost += pCost[th];
        singular = singular || pSingular[th];
    }
    for (int b = 0; b < P; ++b) {
        double g[kP] = {0};
        const size_t go = static_cast<size_t>(b) * kP, dof = static_cast<size_t>(b) * kP * kP;
        for (int th = 0; th < T; ++th) {
            for (int p = 0; p < kP; ++p) g[p] -= pSchur[th][go + p];
            for (int p = 0; p < kP * kP; ++p) o.diag[dof + p] += pDiag[th][dof + p];
        }
        for (int p = 0; p < kP; ++p) o.gradient[go + p] = g[p] - o.directRhs[go + p];
    }
    for (size_t s = 0; s < slots.size(); ++s)
        for (size_t i = 0; i < odim; ++i) o.off[i] += slots[s][i];
    cost += assemblePriors(o);
    // finalizePrimaryDiagonal(1 + damping, 1.0)
    for (int b = 0; b < P; ++b)
        for (int p = 0; p < kP; ++p) {
            double& d = o.diag[static_cast<size_t>(b) * kP * kP + p * kP + p];
            d = d != 0.0 ? d * (1.0 + damping) : 1.0;
        }
    o.lastCost = cost;
    o.lastSingular = singular;
    *costOut = cost;
    *singularOut = singular;
}

struct LinearFailure : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Dense symmetric matrix of the reduced system.
void denseReduced(const Oracle& o, std::vector<double>& A, size_t n) {
    A.assign(n * n, 0.0);
    const int P = o.active.primaryBlockCount;
    for (int b = 0; b < P; ++b)
        for (int i = 0; i < kP; ++i)
            for (int j = 0; j < kP; ++j) A[(b * kP + i) * n + b * kP + j] = o.diag[static_cast<size_t>(b) * kP * kP + i * kP + j];
    for (size_t s = 0; s < o.pairs.size(); ++s) {
        const int r = o.pairs[s].row, c = o.pairs[s].col;
        for (int i = 0; i < kP; ++i)
            for (int j = 0; j < kP; ++j) {
                const double v = o.off[s * kP * kP + i * kP + j];
                A[(r * kP + i) * n + c * kP + j] = v;
                A[(c * kP + j) * n + r * kP + i] = v;
            }
    }
}

bool cholesky(std::vector<double>& A, size_t n) {
    for (size_t j = 0; j < n; ++j) {
        double d = A[j * n + j];
        for (size_t k = 0; k < j; ++k) d -= A[j * n + k] * A[j * n + k];
        if (!(d > 0.0) || !std::isfinite(d)) return false;
        d = std::sqrt(d);
        A[j * n + j] = d;
        const double id = 1.0 / d;
#pragma omp parallel for if (n > 512)
        for (size_t i = j + 1; i < n; ++i) {
            double v = A[i * n + j];
            for (size_t k = 0; k < j; ++k) v -= A[i * n + k] * A[j * n + k];
            A[i * n + j] = v * id;
        }
    }
    return true;
}

void cholSolve(const std::vector<double>& L, size_t n, std::vector<double>& x) {
    for (size_t i = 0; i < n; ++i) {
        double v = x[i];
        for (size_t k = 0; k < i; ++k) v -= L[i * n + k] * x[k];
        x[i] = v / L[i * n + i];
    }
    for (size_t ii = n; ii-- > 0;) {
        double v = x[ii];
        for (size_t k = ii + 1; k < n; ++k) v -= L[k * n + ii] * x[k];
        x[ii] = v / L[ii * n + ii];
    }
}

// Block-sparse y = S x over the 13x13 reduced blocks.
void spmv(const Oracle& o, const std::vector<double>& x, std::vector<double>& y) {
    const int P = o.active.primaryBlockCount;
    std::fill(y.begin(), y.end(), 0.0);
    for (int b = 0; b < P; ++b) {
        const double* D = o.diag.data() + static_cast<size_t>(b) * kP * kP;
        for (int i = 0; i < kP; ++i) {
            double v = 0.0;
            for (int j = 0; j < kP; ++j) v += D[i * kP + j] * x[b * kP + j];
            y[b * kP + i] += v;
        }
    }
    for (size_t s = 0; s < o.pairs.size(); ++s) {
        const int r = o.pairs[s].row, c = o.pairs[s].col;
        const double* B = o.off.data() + s * kP * kP;
        for (int i = 0; i < kP; ++i)
            for (int j = 0; j < kP; ++j) {
                y[r * kP + i] += B[i * kP + j] * x[c * kP + j];
                y[c * kP + j] += B[i * kP + j] * x[r * kP + i];
            }
    }
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

// Linear solve of S x = -g: dense Cholesky or block-Jacobi PCG (stopping rule
// ||r|| <= max(rel * ||b||, abs)).  Both are CPU backends the reference offers
// (BundleAdjustPlaMatrixRuntime.cpp:18-55).
void solveLinear(const Oracle& o, std::vector<double>& x, bool* converged, int* iterations) {
    const int P = o.active.primaryBlockCount;
    const size_t n = static_cast<size_t>(P) * kP;
    std::vector<double> b(n);
    for (size_t i = 0; i < n; ++i) b[i] = -o.gradient[i];
    const double bn = std::sqrt(dot(b, b));
    const double tol = std::max(o.opt.linear_relative_tolerance * bn, o.opt.linear_absolute_tolerance);
    int solver = o.opt.linear_solver;
    if (solver == 0) {
        // a direct solve while the live unknowns fit a dense factor (the reference's CPU backends
        // are direct: dense or sparse Cholesky, BundleAdjustPlaMatrixRuntime.cpp:18-55); the
        // padding columns of the 13-wide blocks carry a unit diagonal (finalizePrimaryDiagonal)
        size_t live = 0;
        for (int blk = 0; blk < P; ++blk)
            for (int p = 0; p < kP; ++p) live += o.diag[static_cast<size_t>(blk) * kP * kP + p * kP + p] != 1.0;
        solver = live <= 8000 ? 1 : 2;
    }
    x.assign(n, 0.0);
    *iterations = 0;
    if (solver == 1) {
        std::vector<double> A;
        denseReduced(o, A, n);
        // the factor runs over the live rows: a padding row is decoupled (zero off-diagonal, unit
        // diagonal, zero right-hand side) and its step is zero
        std::vector<size_t> live;
        for (size_t i = 0; i < n; ++i) {
            bool pad = A[i * n + i] == 1.0 && b[i] == 0.0;
            for (size_t j = 0; j < n && pad; ++j) pad = j == i || A[i * n + j] == 0.0;
            if (!pad) live.push_back(i);
        }
        const size_t m = live.size();
        std::vector<double> Ac(m * m), bc(m);
        for (size_t i = 0; i < m; ++i) {
            bc[i] = b[live[i]];
            for (size_t j = 0; j < m; ++j) Ac[i * m + j] = A[live[i] * n + live[j]];
        }
        std::vector<double> L = Ac;
        if (!cholesky(L, m)) throw LinearFailure("dense Schur matrix is not numerically SPD (positive definite)");
        std::vector<double> xc = bc;
        cholSolve(L, m, xc);
        // direct solve with iterative refinement against the FP64 residual (the reference's direct
        // path keeps a post-solve residual check "after refinement", BundleAdjustPlaMatrix.cpp:
        // 321-330): up to three correction sweeps while |b - S x| exceeds the tolerance
        std::vector<double> res(m);
        double rn = 0.0;
        int sweeps = 0;
        for (;;) {
#pragma omp parallel for if (m > 512)
            for (size_t i = 0; i < m; ++i) {
                double v = bc[i];
                for (size_t j = 0; j < m; ++j) v -= Ac[i * m + j] * xc[j];
                res[i] = v;
            }
            rn = std::sqrt(dot(res, res));
            if (rn <= tol || sweeps == 3) break;
            cholSolve(L, m, res);
            for (size_t i = 0; i < m; ++i) xc[i] += res[i];
            ++sweeps;
        }
        for (size_t i = 0; i < m; ++i) x[live[i]] = xc[i];
        *converged = rn <= tol || !o.opt.residual_gate;
        *iterations = 1 + sweeps;
        return;
    }
    // block-Jacobi preconditioner: Cholesky of each 13x13 diagonal block
    std::vector<std::vector<double>> Lb(P);
    for (int blk = 0; blk < P; ++blk) {
        Lb[blk].assign(o.diag.begin() + static_cast<size_t>(blk) * kP * kP, o.diag.begin() + static_cast<size_t>(blk + 1) * kP * kP);
        if (!cholesky(Lb[blk], kP)) throw LinearFailure("block-Jacobi preconditioner breakdown (not positive definite)");
    }
    auto precond = [&](const std::vector<double>& r, std::vector<double>& z) {
        for (int blk = 0; blk < P; ++blk) {
            std::vector<double> v(r.begin() + blk * kP, r.begin() + (blk + 1) * kP);
            cholSolve(Lb[blk], kP, v);
            std::copy(v.begin(), v.end(), z.begin() + blk * kP);
        }
    };
    const int maxIt = o.opt.max_linear_iterations > 0 ? o.opt.max_linear_iterations : std::max(50, P * 12);
    std::vector<double> r = b, z(n), p(n), q(n);
    precond(r, z);
    p = z;
    double rz = dot(r, z);
    double rn = std::sqrt(dot(r, r));
    *converged = rn <= tol;
    int it = 0;
    while (!*converged && it < maxIt) {
        spmv(o, p, q);
        const double pq = dot(p, q);
        if (!(pq > 0.0) || !std::isfinite(pq)) throw LinearFailure("PCG breakdown");
        const double alpha = rz / pq;
        for (size_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        ++it;
        rn = std::sqrt(dot(r, r));
        if (rn <= tol) {
            // post-solve check of the true residual b - S x (the recursive residual can fall below
            // its FP64 floor near convergence)
            std::vector<double> sx(n);
            spmv(o, x, sx);
            double tr = 0.0;
            for (size_t i = 0; i < n; ++i) tr += (b[i] - sx[i]) * (b[i] - sx[i]);
            *converged = std::sqrt(tr) <= tol || !o.opt.residual_gate;
            break;
        }
        precond(r, z);
        const double rzn = dot(r, z);
        const double beta = rzn / rz;
        rz = rzn;
        for (size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    *iterations = it;
}

// recoverReferencePointSteps (BundleAdjustPlaMatrixReferenceSchur.cpp:982-1082).
void backSubstitute(const Oracle& o, const std::vector<double>& step, std::vector<double>& elim, double* dd, bool* ok) {
    elim.assign(static_cast<size_t>(o.active.trackBlockCount) * kE, 0.0);
    double d = 0.0;
    for (size_t i = 0; i < step.size(); ++i) d += step[i] * o.directRhs[i];
    bool success = true;
    for (size_t t = 0; t < o.nt(); ++t) {
        const int pb = o.active.trackBlock[t];
        if (!o.active.activeTrack[t] || pb < 0) continue;
        const BackSub& bs = o.backSub[t];
        if (!bs.valid) { success = false; continue; }
        double cr[3] = {bs.rhs[0], bs.rhs[1], bs.rhs[2]};
        for (size_t b = 0; b < bs.blocks.size(); ++b) {
            const size_t off = static_cast<size_t>(bs.blocks[b]) * kP;
            for (int e = 0; e < kE; ++e)
                for (int p = 0; p < kP; ++p) cr[e] -= bs.cross[b][p * kE + e] * step[off + p];
        }
        for (int row = 0; row < kE; ++row) {
            double v = 0.0;
            for (int c = 0; c < kE; ++c) v += bs.Vinv[row * kE + c] * cr[c];
            elim[static_cast<size_t>(pb) * kE + row] = v;
            d += bs.rhs[row] * v;
        }
    }
    *dd = d;
    *ok = success;
}

// referenceStepRms (BundleAdjustPlaMatrix.cpp:77-158).
void stepRms(const Oracle& o, const std::vector<double>& ps, const std::vector<double>& es, double* g, double* pt) {
    double gs = 0.0, ss = 0.0;
    size_t gd = 0, sd = 0;
    for (int b = 0; b < o.active.cameraBlockCount; ++b) {
        for (int i = 0; i < 6; ++i) gs += ps[b * kP + i] * ps[b * kP + i];
        gd += 6;
    }
    for (size_t gi = 0; gi < o.state.groups.size(); ++gi) {
        const size_t off = static_cast<size_t>(o.active.cameraBlockCount + static_cast<int>(gi)) * kP;
        for (int p = 0; p < kP; ++p)
            if (o.state.groups[gi].enabled[p]) {
                gs += ps[off + p] * ps[off + p];
                ++gd;
            }
    }
    for (size_t t = 0; t < o.nt(); ++t) {
        const int pb = o.active.trackPrimaryBlock.empty() ? -1 : o.active.trackPrimaryBlock[t];
        if (pb >= 0) {
            for (int i = 0; i < 3; ++i) ss += ps[static_cast<size_t>(pb) * kP + i] * ps[static_cast<size_t>(pb) * kP + i];
            sd += 3;
        }
        const int eb = o.active.trackBlock[t];
        if (eb < 0) continue;
        for (int i = 0; i < 3; ++i) ss += es[eb * 3 + i] * es[eb * 3 + i];
        sd += 3;
    }
    *g = gd ? std::sqrt(gs / gd) : 0.0;
    *pt = sd ? std::sqrt(ss / sd) : 0.0;
}

// applyReferenceCameraPoseStep (BundleAdjustPlaMatrixAssembly.cpp:130-179).
void applyPoseStep(Camera& cam, const double* d) {
    auto mul = [](const double* a, const double* b, double* out) {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double v = 0.0;
                for (int k = 0; k < 3; ++k) v += a[r * 3 + k] * b[k * 3 + c];
                out[r * 3 + c] = v;
            }
    };
    const double sx = std::sin(d[0]), cx = std::cos(d[0]), sy = std::sin(d[1]), cy = std::cos(d[1]);
    const double sz = std::sin(d[2]), cz = std::cos(d[2]);
    const double rx[9] = {1, 0, 0, 0, cx, -sx, 0, sx, cx};
    const double ry[9] = {cy, 0, sy, 0, 1, 0, -sy, 0, cy};
    const double rz[9] = {cz, -sz, 0, sz, cz, 0, 0, 0, 1};
    double t1[9], eul[9];
    mul(rx, ry, t1);
    mul(t1, rz, eul);
    const double sg[3] = {1, -1, -1};
    double tl[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) tl[r * 3 + c] = sg[r] * eul[c * 3 + r] * sg[c];
    double nr[9];
    mul(tl, cam.R, nr);
    std::memcpy(cam.R, nr, sizeof(nr));
    cam.C[0] += d[3];
    cam.C[1] += d[4];
    cam.C[2] += d[5];
}

// The plain parameterisation's pose delta (CameraState::applyDeltaPose,
// BundleAdjustPlaMatrixAssembly.cpp:1134-1136).  The camera library that defines it is not part
// of the reference tree; its first-order form is fixed by the plain rotation columns
// Jw x (X - C) (BundleAdjustPlaMatrixProjection.cpp:208-214), a world-frame rotation vector
// left-multiplied on camera-to-world.  Restated as C2W' = Exp(w) C2W with the exponential summed
// as a power series of the skew matrix (to 1e-20 relative), and C' = C + dC.
void applyPlainPoseStep(Camera& cam, const double* d) {
    const double K[9] = {0.0, -d[2], d[1], d[2], 0.0, -d[0], -d[1], d[0], 0.0};
    double E[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, term[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int n = 1; n < 60; ++n) {
        double nt[9];
        double mx = 0.0;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double v = 0.0;
                for (int k = 0; k < 3; ++k) v += term[r * 3 + k] * K[k * 3 + c];
                nt[r * 3 + c] = v / n;
                mx = std::max(mx, std::fabs(nt[r * 3 + c]));
            }
        std::memcpy(term, nt, sizeof(term));
        for (int i = 0; i < 9; ++i) E[i] += term[i];
        if (mx < 1e-20) break;
    }
    double R[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[r * 3 + c] = E[r * 3] * cam.R[c] + E[r * 3 + 1] * cam.R[3 + c] + E[r * 3 + 2] * cam.R[6 + c];
    std::memcpy(cam.R, R, sizeof(R));
    for (int a = 0; a < 3; ++a) cam.C[a] += d[3 + a];
}

// applyReferenceGaugeTangentStep (BundleAdjustPlaMatrixAssembly.cpp:101-128).
std::array<double, 3> gaugeTangentStep(const Oracle& o, const State& s, double a, double b) {
    const auto origin = targetCoords(s.cams[o.gaugeAnchor].C);
    const auto centre = targetCoords(s.cams[o.gaugeScale].C);
    const auto basis = gaugeBasis(o, s);
    const double td[3] = {basis[0][0] * a + basis[1][0] * b, basis[0][1] * a + basis[1][1] * b,
                          basis[0][2] * a + basis[1][2] * b};
    const std::array<double, 3> dir{centre[0] + td[0] - origin[0], centre[1] + td[1] - origin[1],
                                    centre[2] + td[2] - origin[2]};
    const double len = norm3(dir);
    if (len < 1e-20) return targetCoords(origin.data());
    const double il = 1.0 / len;
    const double out[3] = {origin[0] + dir[0] * il * o.gaugeBaseline, origin[1] + dir[1] * il * o.gaugeBaseline,
                           origin[2] + dir[2] * il * o.gaugeBaseline};
    return targetCoords(out);
}

// applyStep (BundleAdjustPlaMatrixAssembly.cpp:1111-1247) in the reference point
// parameterisation or the plain one (control points), applyIntrinsicStep
// (BundleAdjustPlaMatrixModel.cpp:248-269).
// Rig step (BundleAdjustPlaMatrixAssembly.cpp:1152-1209): placamera::applyPoseDelta on every
// capture and sensor with a block (the plain pose delta, applyPlainPoseStep), then the cameras
// composed again.
void composeRigCamera(const RigPose& cap, const RigPose& sen, Camera& cam) {
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q)
            cam.R[r * 3 + q] = cap.R[r * 3] * sen.R[q] + cap.R[r * 3 + 1] * sen.R[3 + q] + cap.R[r * 3 + 2] * sen.R[6 + q];
    for (int r = 0; r < 3; ++r)
        cam.C[r] = cap.C[r] + cap.R[r * 3] * sen.C[0] + cap.R[r * 3 + 1] * sen.C[1] + cap.R[r * 3 + 2] * sen.C[2];
}

void applyRigPoseStep(RigPose& p, const double* d) {
    Camera tmp{};
    std::memcpy(tmp.R, p.R, sizeof(p.R));
    std::memcpy(tmp.C, p.C, sizeof(p.C));
    applyPlainPoseStep(tmp, d);
    std::memcpy(p.R, tmp.R, sizeof(p.R));
    std::memcpy(p.C, tmp.C, sizeof(p.C));
}

State applyStep(const Oracle& o, const State& s, const std::vector<double>& ps, const std::vector<double>& es,
                double alpha) {
    State n = s;
    const bool ref = o.refParam();
    if (o.hasRig) {
        const Active& a = o.active;
        auto blockOf = [&](const std::vector<int>& index, const std::vector<int>& blocks, size_t i) {
            for (size_t c = 0; c < index.size(); ++c)
                if (index[c] == static_cast<int>(i)) return blocks[c];
            return -1;
        };
        auto step = [&](RigPose& p, int block) {
            if (block < 0) return;
            double d[6];
            for (int i = 0; i < 6; ++i) d[i] = alpha * ps[static_cast<size_t>(block) * kP + i];
            applyRigPoseStep(p, d);
        };
        for (size_t k = 0; k < n.captures.size(); ++k)
            step(n.captures[k], blockOf(a.rigCaptureIndexByCamera, a.rigCaptureBlockByCamera, k));
        for (size_t si = 0; si < n.sensors.size(); ++si)
            step(n.sensors[si], blockOf(a.rigSensorIndexByCamera, a.rigSensorBlockByCamera, si));
        for (size_t c = 0; c < n.cams.size(); ++c)
            composeRigCamera(n.captures[static_cast<size_t>(o.cameraCapture[c])],
                             n.sensors[static_cast<size_t>(o.cameraSensor[c])], n.cams[c]);
    }
    for (size_t c = 0; c < n.cams.size() && !o.hasRig; ++c) {
        const int b = o.active.cameraBlock[c];
        if (b < 0) continue;
        double d[6];
        for (int i = 0; i < 6; ++i) d[i] = alpha * ps[static_cast<size_t>(b) * kP + i];
        if (!ref) {
            applyPlainPoseStep(n.cams[c], d);
        } else if (usesGaugeTangent(o, c)) {
            const auto centre = gaugeTangentStep(o, n, d[3], d[4]);
            const double rd[6] = {d[0], d[1], d[2], 0, 0, 0};
            applyPoseStep(n.cams[c], rd);
            n.cams[c].C[0] = centre[0];
            n.cams[c].C[1] = centre[1];
            n.cams[c].C[2] = centre[2];
        } else {
            applyPoseStep(n.cams[c], d);
        }
    }
    for (size_t g = 0; g < n.groups.size(); ++g) {
        Group& gr = n.groups[g];
        const size_t off = static_cast<size_t>(o.active.cameraBlockCount + static_cast<int>(g)) * kP;
        for (int p = 0; p < kP; ++p)
            if (gr.enabled[p]) gr.params[p] = std::clamp(gr.params[p] + alpha * ps[off + p], gr.lower[p], gr.upper[p]);
    }
    for (size_t t = 0; t < n.points.size(); ++t) {
        const int pb = o.active.trackPrimaryBlock.empty() ? -1 : o.active.trackPrimaryBlock[t];
        if (pb >= 0) {
            // a promoted point: the primary step (the plain parameterisation)
            for (int a = 0; a < 3; ++a) n.points[t][a] += alpha * ps[static_cast<size_t>(pb) * kP + a];
            continue;
        }
        const int eb = o.active.trackBlock[t];
        if (eb < 0) continue;
        const double sc = ref ? referencePointScale(s.points[t].data()) : 1.0;
        for (int a = 0; a < 3; ++a) n.points[t][a] += sc * alpha * es[static_cast<size_t>(eb) * 3 + a];
    }
    return n;
}

// evaluateObjective (BundleAdjustPlaMatrixAssembly.cpp:1010-1019): image and control-point
// costs of the active tracks (:674-690) plus intrinsic priors; an invalid projection makes the cost +inf
// (BundleAdjustPlaMatrix.cpp:42-58).
double objective(const Oracle& o, const State& s) {
    const int T = std::max(1, std::min<int>(o.threads, static_cast<int>(o.nt())));
    std::vector<Camera> eff(s.cams.size());
    for (size_t c = 0; c < s.cams.size(); ++c) eff[c] = effectiveCamera(o, s, c);
    std::vector<double> part(T, 0.0);
    std::vector<char> bad(T, 0);
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int th = 0; th < T; ++th) {
        double cost = 0.0;
        for (size_t t = o.boundaries[th]; t < o.boundaries[th + 1] && !bad[th]; ++t) {
            if (!o.active.activeTrack[t]) continue;
            for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k) {
                const Obs& ob = o.obs[k];
                if (!obsUsable(ob, s.cams.size())) continue;
                ProjectionDerivatives pd;
                if (!projectFull(eff[ob.cam], s.points[t].data(), &pd, false)) { bad[th] = 1; break; }
                const double rx = pd.px[0] - ob.u, ry = pd.px[1] - ob.v;
                const double ms = sanitizedScale(ob);
                const double w = sanitizedWeight(ob) / (ms * ms);
                RobustEval rb;
                if (!robustLoss(w * (rx * rx + ry * ry), o.opt.robust_loss, o.opt.robust_loss_scale, &rb) ||
                    !std::isfinite(rb.cost)) {
                    bad[th] = 1;
                    break;
                }
                cost += rb.cost;
            }
            if (bad[th]) break;
            for (const auto& cp : o.controlPoints[t]) {
                double r[3];
                RobustEval rb;
                if (controlPointResidual(o, cp, s.points[t].data(), r, &rb)) cost += rb.cost;
            }
        }
        part[th] = cost;
    }
    double cost = 0.0;
    for (int th = 0; th < T; ++th) {
        if (bad[th]) return kInf;
        cost += part[th];
    }
    cost += priorCost(o, s);
    // assembleScaleBars (BundleAdjustPlaMatrixAssemblySurvey.cpp:131-186): bars of active tracks
    for (const auto& sb : o.scaleBars) {
        if (!o.active.activeTrack[sb.a] || !o.active.activeTrack[sb.b]) continue;
        double r, J[3];
        RobustEval rb;
        if (scaleBarResidual(o, sb, s.points[sb.a].data(), s.points[sb.b].data(), &r, J, &rb)) cost += rb.cost;
    }
    return cost;
}

// strictTrackRms (BundleAdjustQuality.cpp:302-364).
double strictTrackRms(const Oracle& o, const std::vector<Camera>& cams, size_t t, const double* X) {
    if (!std::isfinite(X[0]) || !std::isfinite(X[1]) || !std::isfinite(X[2])) return kInf;
    double sum = 0.0;
    int count = 0, first = -1;
    bool second = false;
    for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k) {
        const Obs& ob = o.obs[k];
        double w = sanitizedWeight(ob);
        const double sc = sanitizedScale(ob);
        w /= sc * sc;
        if (!(w > 0.0)) continue;
        if (ob.cam < 0 || ob.cam >= static_cast<int>(cams.size()) || !std::isfinite(ob.u) || !std::isfinite(ob.v))
            return kInf;
        ProjectionDerivatives pd;
        if (!projectFull(cams[ob.cam], X, &pd, false)) return kInf;
        const double du = pd.px[0] - ob.u, dv = pd.px[1] - ob.v;
        sum += w * (du * du + dv * dv);
        count += 2;
        if (first < 0) first = ob.cam;
        else if (ob.cam != first) second = true;
    }
    if (count < 4 || !second) return kInf;
    return std::sqrt(sum / count);
}

// publishIntrinsics (BundleAdjustPlaMatrixModel.cpp:271-352): refined cameras carry the group
// intrinsics.
std::vector<Camera> publishCameras(const Oracle& o, const State& s) {
    std::vector<Camera> out = s.cams;
    if (s.groups.empty()) return out;
    const auto& refs = o.refCams.empty() ? o.inputCams : o.refCams;
    for (size_t c = 0; c < out.size(); ++c) {
        const Group& g = s.groups[static_cast<size_t>(o.active.calibGroupByCamera[c])];
        const Camera& src = o.inputCams[c];
        const double focal = g.enabled[0] ? g.params[0] : src.fx;
        const double aspect = g.enabled[1] ? std::exp(g.params[1]) : src.fy / src.fx;
        out[c].fx = focal;
        out[c].fy = focal * std::exp(std::log(aspect));
        out[c].cx = g.enabled[2] ? refs[c].cx + g.params[2] : src.cx;
        out[c].cy = g.enabled[3] ? refs[c].cy + g.params[3] : src.cy;
        double* dist[5] = {&out[c].k1, &out[c].k2, &out[c].k3, &out[c].p1, &out[c].p2};
        const double srcd[5] = {src.k1, src.k2, src.k3, src.p1, src.p2};
        for (int p = 4; p < 9; ++p) *dist[p - 4] = g.enabled[p] ? g.params[p] : srcd[p - 4];
    }
    return out;
}

// ---- General (non-online) path ----------------------------------------------------------------
// The reference's default path (useReferenceOnlineSchur = false, include/plabundle/options.h:65):
// buildNormalEquations assembles undamped block normal equations once per linearisation
// (BundleAdjustPlaMatrixAssembly.cpp:586-939) and solveDampedSchurComplement (PlaMatrix, absent
// from the tree) eliminates the points and solves (call site BundleAdjustPlaMatrix.cpp:311-357).
//
// BlockNormalEquations<double> restated from its use sites: a residual block r with Jacobians J_b
// (rows x block size) and weight w adds H_bc += w J_b^T J_c and g_b += w J_b^T r over all pairs of
// its blocks.  Primary blocks are 13 wide, eliminated blocks 3.
struct GeneralEquations {
    int P = 0, E = 0;
    std::vector<double> diag, gp, hee, ge;                    // P*13*13, P*13, E*9, E*3
    std::map<std::pair<int, int>, std::vector<double>> off;  // (row < col) -> 13 x 13
    std::map<std::pair<int, int>, std::vector<double>> cpl;  // (eliminated, primary) -> 13 x 3
    void reset(int p, int e) {
        P = p;
        E = e;
        diag.assign(static_cast<size_t>(P) * kP * kP, 0.0);
        gp.assign(static_cast<size_t>(P) * kP, 0.0);
        hee.assign(static_cast<size_t>(E) * 9, 0.0);
        ge.assign(static_cast<size_t>(E) * 3, 0.0);
        off.clear();
        cpl.clear();
    }
    // addResidualBlocks(primary, Jp, n, eliminated, Je, r, rows, w) (...Assembly.cpp:413-421);
    // eliminated < 0: addPrimaryResidualBlocks; n == 0: addEliminatedResidualBlock.  Every ordered
    // pair of terms (a, b) adds J_a^T J_b to block (prim a, prim b); the stored upper block takes
    // the pairs with prim a < prim b, the diagonal block those with prim a == prim b.
    void addResidualBlocks(const int* prim, const double* const* Jp, int n, int elim, const double* Je,
                           const double* r, int rows, double w) {
        for (int a = 0; a < n; ++a) {
            for (int i = 0; i < kP; ++i) {
                double s = 0.0;
                for (int k = 0; k < rows; ++k) s += Jp[a][k * kP + i] * r[k];
                gp[static_cast<size_t>(prim[a]) * kP + i] += w * s;
            }
            for (int b = 0; b < n; ++b) {
                if (prim[a] > prim[b]) continue;
                double* dst;
                if (prim[a] == prim[b]) {
                    dst = diag.data() + static_cast<size_t>(prim[a]) * kP * kP;
                } else {
                    auto& blk = off[{prim[a], prim[b]}];
                    if (blk.empty()) blk.assign(kP * kP, 0.0);
                    dst = blk.data();
                }
                for (int i = 0; i < kP; ++i)
                    for (int j = 0; j < kP; ++j) {
                        double s = 0.0;
                        for (int k = 0; k < rows; ++k) s += Jp[a][k * kP + i] * Jp[b][k * kP + j];
                        dst[i * kP + j] += w * s;
                    }
            }
            if (elim >= 0) {
                auto& blk = cpl[{elim, prim[a]}];
                if (blk.empty()) blk.assign(kP * kE, 0.0);
                for (int i = 0; i < kP; ++i)
                    for (int j = 0; j < kE; ++j) {
                        double s = 0.0;
                        for (int k = 0; k < rows; ++k) s += Jp[a][k * kP + i] * Je[k * kE + j];
                        blk[i * kE + j] += w * s;
                    }
            }
        }
        if (elim >= 0) {
            for (int i = 0; i < kE; ++i) {
                double s = 0.0;
                for (int k = 0; k < rows; ++k) s += Je[k * kE + i] * r[k];
                ge[static_cast<size_t>(elim) * 3 + i] += w * s;
                for (int j = 0; j < kE; ++j) {
                    double h = 0.0;
                    for (int k = 0; k < rows; ++k) h += Je[k * kE + i] * Je[k * kE + j];
                    hee[static_cast<size_t>(elim) * 9 + i * 3 + j] += w * h;
                }
            }
        }
    }
};

// buildNormalEquations (BundleAdjustPlaMatrixAssembly.cpp:586-939) at the current state for frame
// cameras: every usable observation of an active track through addObservation (:381-440): its
// primary terms (camera pose block, intrinsic group block) and the track's eliminated point;
// control points through addPointResidual (:356-380, :663-672); the intrinsic priors through
// assemblePrimaryPriors (AssemblySurvey.cpp:43-91, weight 1).  Returns the linearised cost.
double buildGeneral(Oracle& o, GeneralEquations& q) {
    q.reset(o.active.primaryBlockCount, o.active.trackBlockCount);
    const bool ref = o.refParam();
    double cost = 0.0;
    for (size_t t = 0; t < o.nt(); ++t) {
        if (!o.active.activeTrack[t]) continue;
        const int elim = o.active.trackBlock[t];
        const int prim = o.active.trackPrimaryBlock[t];
        for (int64_t k = o.offs[t]; k < o.offs[t + 1]; ++k) {
            const Obs& ob = o.obs[k];
            if (!obsUsable(ob, o.state.cams.size())) continue;
            const Camera cam = effectiveCamera(o, o.state, ob.cam);
            Lin L;
            if (!linearize(cam, activeIntrinsics(o, ob.cam), o.state.points[t].data(), ob, o.opt.robust_loss,
                           o.opt.robust_loss_scale, ref, &L))
                throw InvalidProjection("linearisation produced an invalid projection");
            cost += L.cost;
            const Terms tm = primaryTerms(o, o.state, ob.cam, L);
            int blocks[4] = {tm.blocks[0], tm.blocks[1], tm.blocks[2], -1};
            const double* jp[4] = {tm.J[0], tm.J[1], tm.J[2], nullptr};
            int count = tm.count;
            double Jpp[2 * kP] = {0};
            if (prim >= 0) {
                // addObservation's point primary term: the point Jacobian padded to 13 columns
                for (int k = 0; k < 2; ++k)
                    for (int c = 0; c < 3; ++c) Jpp[k * kP + c] = L.Jp[k * kE + c];
                blocks[count] = prim;
                jp[count++] = Jpp;
            }
            q.addResidualBlocks(blocks, jp, count, elim, L.Jp, L.r, 2, L.nw);
        }
        for (const auto& cp : o.controlPoints[t]) {
            double r[3];
            RobustEval rb;
            if (!controlPointResidual(o, cp, o.state.points[t].data(), r, &rb)) continue;
            cost += rb.cost;
            if (elim >= 0) {
                q.addResidualBlocks(nullptr, nullptr, 0, elim, cp.J, r, 3, rb.weight);
            } else if (prim >= 0) {
                // addPointResidual on a primary point block (BundleAdjustPlaMatrixAssembly.cpp:356-380)
                double Jc[3 * kP] = {0};
                for (int k = 0; k < 3; ++k)
                    for (int c = 0; c < 3; ++c) Jc[k * kP + c] = cp.J[k * 3 + c];
                const double* jc[1] = {Jc};
                q.addResidualBlocks(&prim, jc, 1, -1, nullptr, r, 3, rb.weight);
            }
        }
    }
    // assembleScaleBars (BundleAdjustPlaMatrixAssemblySurvey.cpp:131-186)
    for (const auto& sb : o.scaleBars) {
        if (!o.active.activeTrack[sb.a] || !o.active.activeTrack[sb.b]) continue;
        double r, J[3];
        RobustEval rb;
        if (!scaleBarResidual(o, sb, o.state.points[sb.a].data(), o.state.points[sb.b].data(), &r, J, &rb)) continue;
        cost += rb.cost;
        double Ja[kP] = {0}, Jb[kP] = {0};
        for (int c = 0; c < 3; ++c) {
            Ja[c] = J[c];
            Jb[c] = -J[c];
        }
        int blocks[2];
        const double* jp[2];
        int count = 0;
        if (o.active.trackPrimaryBlock[sb.a] >= 0) {
            blocks[count] = o.active.trackPrimaryBlock[sb.a];
            jp[count++] = Ja;
        }
        if (o.active.trackPrimaryBlock[sb.b] >= 0) {
            blocks[count] = o.active.trackPrimaryBlock[sb.b];
            jp[count++] = Jb;
        }
        if (count > 0) q.addResidualBlocks(blocks, jp, count, -1, nullptr, &r, 1, rb.weight);
    }
    for (size_t g = 0; g < o.state.groups.size(); ++g) {
        const Group& gr = o.state.groups[g];
        const int block = o.active.cameraBlockCount + static_cast<int>(g);
        std::vector<double> J(kP * kP, 0.0), r(kP, 0.0);
        for (int p = 0; p < kP; ++p) {
            if (!gr.enabled[p]) continue;
            r[p] = gr.invSigma[p] * (gr.params[p] - gr.prior[p]);
            J[p * kP + p] = gr.invSigma[p];
            cost += 0.5 * r[p] * r[p];
        }
        const double* jp[1] = {J.data()};
        q.addResidualBlocks(&block, jp, 1, -1, nullptr, r.data(), kP, 1.0);
    }
    return cost;
}

// solveDampedSchurComplement restated (PlaMatrix is absent; the damping form is the online path's,
// BundleAdjustPlaMatrixReferenceSchur.cpp:362-365, :930): primary and eliminated diagonals times
// (1 + damping), a zero primary diagonal entry set to 1; S = H_pp - sum W V^-1 W^T,
// b = -g_p + sum W V^-1 g_e; dense FP64 Cholesky; y_e = V^-1 (-g_e - W^T x).  `converged`: the
// residual |b - S x| is within max(tol |b|, 1e-12).
void solveGeneralDamped(const GeneralEquations& q, double damping, double tol, bool gate, std::vector<double>& x,
                        std::vector<double>& y, bool* converged) {
    const size_t n = static_cast<size_t>(q.P) * kP;
    std::vector<double> S(n * n, 0.0), b(n);
    for (int blk = 0; blk < q.P; ++blk)
        for (int i = 0; i < kP; ++i)
            for (int j = 0; j < kP; ++j) {
                double v = q.diag[static_cast<size_t>(blk) * kP * kP + i * kP + j];
                if (i == j) v = v != 0.0 ? v * (1.0 + damping) : 1.0;
                S[(static_cast<size_t>(blk) * kP + i) * n + static_cast<size_t>(blk) * kP + j] = v;
            }
    for (const auto& kv : q.off) {
        const size_t r0 = static_cast<size_t>(kv.first.first) * kP, c0 = static_cast<size_t>(kv.first.second) * kP;
        for (int i = 0; i < kP; ++i)
            for (int j = 0; j < kP; ++j) {
                S[(r0 + i) * n + c0 + j] = kv.second[i * kP + j];
                S[(c0 + j) * n + r0 + i] = kv.second[i * kP + j];
            }
    }
    for (size_t i = 0; i < n; ++i) b[i] = -q.gp[i];
    std::vector<std::array<double, 9>> inv(q.E);
    for (int e = 0; e < q.E; ++e) {
        double V[9];
        for (int i = 0; i < 9; ++i) V[i] = q.hee[static_cast<size_t>(e) * 9 + i];
        for (int d = 0; d < 3; ++d) V[d * 4] *= 1.0 + damping;
        if (!inverse3x3(V, inv[e].data(), 1.0e-15)) throw LinearFailure("eliminated block is not numerically SPD");
    }
    // couplings of each eliminated block (the map is ordered by eliminated block)
    auto it = q.cpl.begin();
    while (it != q.cpl.end()) {
        const int e = it->first.first;
        std::vector<std::pair<int, const std::vector<double>*>> ws;
        while (it != q.cpl.end() && it->first.first == e) {
            ws.push_back({it->first.second, &it->second});
            ++it;
        }
        const auto& iv = inv[e];
        std::vector<std::vector<double>> Y(ws.size(), std::vector<double>(kP * kE, 0.0));
        for (size_t a = 0; a < ws.size(); ++a)
            for (int i = 0; i < kP; ++i)
                for (int k = 0; k < kE; ++k)
                    for (int m = 0; m < kE; ++m) Y[a][i * kE + k] += (*ws[a].second)[i * kE + m] * iv[m * 3 + k];
        for (size_t a = 0; a < ws.size(); ++a) {
            const size_t ra = static_cast<size_t>(ws[a].first) * kP;
            for (int i = 0; i < kP; ++i)
                for (int k = 0; k < kE; ++k) b[ra + i] += Y[a][i * kE + k] * q.ge[static_cast<size_t>(e) * 3 + k];
            for (size_t c = 0; c < ws.size(); ++c) {
                const size_t rc = static_cast<size_t>(ws[c].first) * kP;
                for (int i = 0; i < kP; ++i)
                    for (int j = 0; j < kP; ++j) {
                        double h = 0.0;
                        for (int k = 0; k < kE; ++k) h += Y[a][i * kE + k] * (*ws[c].second)[j * kE + k];
                        S[(ra + i) * n + rc + j] -= h;
                    }
            }
        }
    }
    std::vector<double> L = S;
    if (!cholesky(L, n)) throw LinearFailure("dense Schur matrix is not numerically SPD (positive definite)");
    x = b;
    cholSolve(L, n, x);
    // iterative refinement against the FP64 residual, up to three sweeps (as the online path's
    // direct solve)
    double bn = 0.0;
    for (size_t i = 0; i < n; ++i) bn += b[i] * b[i];
    const double limit = std::max(tol * std::sqrt(bn), 1.0e-12);
    std::vector<double> res(n);
    double rn = 0.0;
    for (int sweep = 0;; ++sweep) {
        rn = 0.0;
        for (size_t i = 0; i < n; ++i) {
            double v = b[i];
            for (size_t j = 0; j < n; ++j) v -= S[i * n + j] * x[j];
            res[i] = v;
            rn += v * v;
        }
        if (std::sqrt(rn) <= limit || sweep == 3) break;
        cholSolve(L, n, res);
        for (size_t i = 0; i < n; ++i) x[i] += res[i];
    }
    *converged = std::sqrt(rn) <= limit || !gate;
    std::vector<double> r(static_cast<size_t>(q.E) * 3);
    for (int e = 0; e < q.E; ++e)
        for (int k = 0; k < 3; ++k) r[static_cast<size_t>(e) * 3 + k] = -q.ge[static_cast<size_t>(e) * 3 + k];
    for (const auto& kv : q.cpl) {
        const int e = kv.first.first;
        const size_t ra = static_cast<size_t>(kv.first.second) * kP;
        for (int k = 0; k < kE; ++k)
            for (int i = 0; i < kP; ++i) r[static_cast<size_t>(e) * 3 + k] -= kv.second[i * kE + k] * x[ra + i];
    }
    y.assign(static_cast<size_t>(q.E) * 3, 0.0);
    for (int e = 0; e < q.E; ++e)
        for (int k = 0; k < 3; ++k) {
            double v = 0.0;
            for (int m = 0; m < 3; ++m) v += inv[e][k * 3 + m] * r[static_cast<size_t>(e) * 3 + m];
            y[static_cast<size_t>(e) * 3 + k] = v;
        }
}

// The general branch of optimizePointsWithPlaMatrix (BundleAdjustPlaMatrix.cpp:236-542 with
// use_reference_online_schur false): one buildNormalEquations per accepted state, damped solves
// to 1e-12 (retried with ten times the damping at the same state when short of the tolerance or
// rejected), convergence when the step RMS is at most 1e-6 before a line search, a forward-
// difference directional decrease (step 1e-4), Armijo with the general path's limit, and the
// last (smallest) trial accepted when it lowers the cost.  A solver breakdown is a numerical
// failure.
void solveGeneralPath(Oracle* o, orc_report* rep, double* current_out, int* iterations_out, bool* converged_out,
                      bool* failed_out) {
    const Active& a = o->active;
    const int T = std::max(1, std::min<int>(o->threads, static_cast<int>(o->nt())));
    trackBoundaries(*o, T);
    double current = std::numeric_limits<double>::quiet_NaN(), damping = 0.0;
    int iterations = 0;
    bool converged = a.primaryBlockCount == 0 && a.trackBlockCount == 0;
    bool failed = false;
    GeneralEquations q;
    std::vector<double> ps, es;
    const double tol = o->opt.linear_relative_tolerance > 0 ? o->opt.linear_relative_tolerance : 1.0e-12;
    try {
        if (converged) {
            current = objective(*o, o->state);
            rep->initial_cost = current;
            ++rep->objective_evaluations;
        }
        const int budget = std::max(1, o->opt.max_iterations);
        while (iterations < budget && !converged) {
            const auto ta = std::chrono::steady_clock::now();
            current = buildGeneral(*o, q);
            rep->assembly_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count();
            ++rep->linearizations;
            ++rep->objective_evaluations;
            if (rep->linearizations == 1) rep->initial_cost = current;
            bool relinearize = false;
            while (iterations < budget && !converged && !relinearize) {
                bool lconv = false;
                const auto tl = std::chrono::steady_clock::now();
                solveGeneralDamped(q, damping, tol, o->opt.residual_gate != 0, ps, es, &lconv);
                rep->linear_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - tl).count();
                rep->linear_iterations += 1;
                ++iterations;
                if (!lconv) {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                double rg = 0.0, rp = 0.0;
                stepRms(*o, ps, es, &rg, &rp);
                if (rg <= 1e-6 && rp <= 1e-6) {
                    converged = true;
                    continue;
                }
                double dd = 0.0;
                {
                    const double h = 1.0e-4;
                    const State fs = applyStep(*o, o->state, ps, es, h);
                    const double fd = objective(*o, fs);
                    ++rep->objective_evaluations;
                    if (std::isfinite(fd) && fd < current) dd = (current - fd) / h;
                }
                double cand = kInf, alpha = 1.0, tried = 1.0;
                bool armijo = false;
                State cs;
                for (int ls = 0; ls < o->opt.line_search_steps; ++ls) {
                    cs = applyStep(*o, o->state, ps, es, alpha);
                    cand = objective(*o, cs);
                    tried = alpha;
                    ++rep->objective_evaluations;
                    const double limit = dd > 0.0 ? current - o->opt.armijo_coefficient * alpha * dd : current;
                    if (std::isfinite(cand) && cand <= limit && cand < current) {
                        armijo = true;
                        break;
                    }
                    alpha *= 0.5;
                }
                (void)armijo;
                const bool accept = std::isfinite(cand) && cand < current;
                if (std::getenv("PB_GPU_TRACE"))
                    std::fprintf(stderr,
                                 "ORACLE_TRACE general it=%d cost=%.15e lambda=%.3e dd=%.6e rms_global=%.3e "
                                 "rms_point=%.3e alpha=%.6g cand=%.15e accepted=%d\n",
                                 iterations, current, damping, dd, rg, rp, tried, cand, accept ? 1 : 0);
                if (accept) {
                    o->state = std::move(cs);
                    current = cand;
                    ++rep->accepted_steps;
                    damping /= 10.0;
                    converged = tried * rg <= 1e-6 && tried * rp <= 1e-6;
                    relinearize = !converged;
                } else {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                }
            }
        }
    } catch (const std::exception&) {
        failed = true;
    }
    *current_out = current;
    *iterations_out = iterations;
    *converged_out = converged;
    *failed_out = failed;
}

}  // namespace orc

using namespace orc;

extern "C" {

// Rig topology (Problem::rig): composeRigCameras replaces every camera's pose by the composition of
// its capture and sensor, R = R_rig R_sensor and C = C_rig + R_rig c_sensor (runConcreteBackend,
// src/solver.cpp:282; the composition is stated in the reference's README, "Rig BA"); without
// explicit calibration groups the cameras of one sensor share a group (makeSolverOptions,
// Conversion.cpp:83-98); a camera whose capture and sensor are both fixed becomes a fixed camera
// (:120-142).  The camera library that validates the topology is absent from the reference tree;
// its checks are restated as: bindings to existing records of the same rig, proper rotations,
// finite centres, a fixed sensor in every rig.
int loadRig(Oracle& o, const orc_problem* pr) {
    if (pr->n_rig_captures <= 0) return 0;
    const int nc = static_cast<int>(o.inputCams.size());
    if (pr->n_rig_sensors <= 0 || !pr->rig_captures || !pr->rig_capture_info || !pr->rig_sensors ||
        !pr->rig_sensor_info || !pr->rig_camera_capture || !pr->rig_camera_sensor)
        return InvalidInput;
    auto properRotation = [](const double* R) {
        for (int i = 0; i < 9; ++i)
            if (!std::isfinite(R[i])) return false;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double v = 0.0;
                for (int k = 0; k < 3; ++k) v += R[r * 3 + k] * R[c * 3 + k];
                if (std::fabs(v - (r == c ? 1.0 : 0.0)) > 1e-9) return false;
            }
        const double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                           R[2] * (R[3] * R[7] - R[4] * R[6]);
        return std::fabs(det - 1.0) <= 1e-9;
    };
    auto load = [&](const double* rec, int n, std::vector<RigPose>& out) {
        out.resize(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) {
            std::memcpy(out[i].R, rec + static_cast<size_t>(i) * 12, 9 * sizeof(double));
            std::memcpy(out[i].C, rec + static_cast<size_t>(i) * 12 + 9, 3 * sizeof(double));
            if (!properRotation(out[i].R) || !std::isfinite(out[i].C[0]) || !std::isfinite(out[i].C[1]) ||
                !std::isfinite(out[i].C[2]))
                return false;
        }
        return true;
    };
    if (!load(pr->rig_captures, pr->n_rig_captures, o.inputCaptures)) return InvalidInput;
    if (!load(pr->rig_sensors, pr->n_rig_sensors, o.inputSensors)) return InvalidInput;
    o.captureInfo.assign(pr->rig_capture_info, pr->rig_capture_info + 2 * pr->n_rig_captures);
    o.sensorInfo.assign(pr->rig_sensor_info, pr->rig_sensor_info + 2 * pr->n_rig_sensors);
    o.cameraCapture.assign(pr->rig_camera_capture, pr->rig_camera_capture + nc);
    o.cameraSensor.assign(pr->rig_camera_sensor, pr->rig_camera_sensor + nc);
    for (int c = 0; c < nc; ++c) {
        const int k = o.cameraCapture[c], si = o.cameraSensor[c];
        if (k < 0 || k >= pr->n_rig_captures || si < 0 || si >= pr->n_rig_sensors) return InvalidInput;
        if (o.captureInfo[2 * k] != o.sensorInfo[2 * si]) return InvalidInput;
    }
    for (int k = 0; k < pr->n_rig_captures; ++k) {
        bool fixedSensor = false;
        for (int si = 0; si < pr->n_rig_sensors; ++si)
            fixedSensor = fixedSensor || (o.sensorInfo[2 * si] == o.captureInfo[2 * k] && o.sensorInfo[2 * si + 1] != 0);
        if (!fixedSensor) return InvalidInput;
    }
    o.hasRig = true;
    for (int c = 0; c < nc; ++c)
        composeRigCamera(o.inputCaptures[o.cameraCapture[c]], o.inputSensors[o.cameraSensor[c]], o.inputCams[c]);
    if (o.groupIds.empty()) o.groupIds = o.cameraSensor;
    for (int c = 0; c < nc; ++c)
        if (o.captureInfo[2 * o.cameraCapture[c] + 1] && o.sensorInfo[2 * o.cameraSensor[c] + 1] &&
            std::find(o.fixedCams.begin(), o.fixedCams.end(), c) == o.fixedCams.end())
            o.fixedCams.push_back(c);
    return 0;
}

void* orc_create(const orc_problem* pr, const orc_options* op, int32_t* status) {
    auto o = std::make_unique<Oracle>();
    o->opt = *op;
    o->inputCams.resize(static_cast<size_t>(pr->n_cameras));
    for (int c = 0; c < pr->n_cameras; ++c) o->inputCams[c] = loadCamera(pr->cameras + static_cast<size_t>(c) * ORC_CAMERA_STRIDE);
    if (pr->intrinsic_reference_cameras) {
        o->refCams.resize(o->inputCams.size());
        for (int c = 0; c < pr->n_cameras; ++c)
            o->refCams[c] = loadCamera(pr->intrinsic_reference_cameras + static_cast<size_t>(c) * ORC_CAMERA_STRIDE);
    }
    o->offs.assign(pr->track_offsets, pr->track_offsets + pr->n_tracks + 1);
    o->initialPoints.resize(static_cast<size_t>(pr->n_tracks));
    for (int t = 0; t < pr->n_tracks; ++t)
        for (int a = 0; a < 3; ++a) o->initialPoints[t][a] = pr->points[static_cast<size_t>(t) * 3 + a];
    o->obs.resize(static_cast<size_t>(pr->n_obs));
    for (int64_t k = 0; k < pr->n_obs; ++k)
        o->obs[k] = {pr->obs_camera[k], pr->obs_u[k], pr->obs_v[k], pr->obs_weight[k], pr->obs_scale[k]};
    o->fixedCams.assign(pr->fixed_cameras, pr->fixed_cameras + pr->n_fixed_cameras);
    o->fixedTracks.assign(pr->fixed_tracks, pr->fixed_tracks + pr->n_fixed_tracks);
    if (pr->calibration_group_ids) o->groupIds.assign(pr->calibration_group_ids, pr->calibration_group_ids + pr->n_cameras);
#ifdef _OPENMP
    o->threads = op->num_threads > 0 ? op->num_threads : omp_get_max_threads();
#else
    o->threads = 1;
#endif
    int st = 0;
    if (o->inputCams.empty() || o->nt() == 0) st = InvalidInput;
    if (!st) st = loadRig(*o, pr);
    if (!st) st = loadControlPoints(*o, pr);
    if (!st) st = loadScaleBars(*o, pr);
    // a problem with scale bars has no online path (canUseReferenceOnlineSchur)
    if (!st && !o->scaleBars.empty()) o->opt.general_path = 1;
    if (!st) st = normalizeGauge(*o);
    if (!st) {
        prepareActive(*o);
        o->state.cams = o->inputCams;
        o->state.points = o->initialPoints;
        o->state.captures = o->inputCaptures;
        o->state.sensors = o->inputSensors;
        initGroups(*o);
        trackBoundaries(*o, std::max(1, std::min<int>(o->threads, static_cast<int>(o->nt()))));
    }
    *status = st;
    return o.release();
}

void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

int32_t orc_rig(void* h, double* captures, double* sensors, int32_t* capture_block, int32_t* sensor_block) {
    auto* o = static_cast<Oracle*>(h);
    if (!o->hasRig) return InvalidInput;
    const Active& a = o->active;
    for (size_t k = 0; k < o->state.captures.size(); ++k) {
        if (captures) {
            std::memcpy(captures + k * 12, o->state.captures[k].R, 9 * sizeof(double));
            std::memcpy(captures + k * 12 + 9, o->state.captures[k].C, 3 * sizeof(double));
        }
        if (capture_block) {
            capture_block[k] = -1;
            for (size_t c = 0; c < o->inputCams.size(); ++c)
                if (a.rigCaptureIndexByCamera[c] == static_cast<int>(k)) capture_block[k] = a.rigCaptureBlockByCamera[c];
        }
    }
    for (size_t si = 0; si < o->state.sensors.size(); ++si) {
        if (sensors) {
            std::memcpy(sensors + si * 12, o->state.sensors[si].R, 9 * sizeof(double));
            std::memcpy(sensors + si * 12 + 9, o->state.sensors[si].C, 3 * sizeof(double));
        }
        if (sensor_block) {
            sensor_block[si] = -1;
            for (size_t c = 0; c < o->inputCams.size(); ++c)
                if (a.rigSensorIndexByCamera[c] == static_cast<int>(si)) sensor_block[si] = a.rigSensorBlockByCamera[c];
        }
    }
    return 0;
}

int32_t orc_control_point_whitening(const double* record, double* W) { return controlPointWhitening(record, W) ? 1 : 0; }

int32_t orc_info(void* h, int32_t* counts, double* baseline) {
    auto* o = static_cast<Oracle*>(h);
    counts[0] = o->active.primaryBlockCount;
    counts[1] = o->active.cameraBlockCount;
    counts[2] = o->active.intrinsicBlockCount;
    counts[3] = o->active.trackBlockCount;
    counts[4] = o->active.activeTrackCount;
    counts[5] = o->active.observationCount;
    counts[6] = o->active.rejectedInitialTracks;
    counts[7] = static_cast<int32_t>(o->pairs.size());
    counts[8] = o->gaugeAnchor;
    counts[9] = o->gaugeScale;
    counts[10] = static_cast<int32_t>(o->fixedCams.size());
    counts[11] = o->fixedCams.empty() ? -1 : o->fixedCams.front();
    counts[12] = o->refParam() ? 1 : 0;
    *baseline = o->gaugeBaseline;
    return 0;
}

int32_t orc_active(void* h, int8_t* at, int32_t* cb, int32_t* ib, int32_t* tb) {
    auto* o = static_cast<Oracle*>(h);
    for (size_t t = 0; t < o->nt(); ++t) {
        at[t] = o->active.activeTrack[t];
        tb[t] = o->active.trackBlock[t];
    }
    for (size_t c = 0; c < o->inputCams.size(); ++c) {
        cb[c] = o->active.cameraBlock[c];
        ib[c] = o->active.intrinsicBlockByCamera[c];
    }
    return 0;
}

int32_t orc_linearize_observations(void* h, double* res, double* jp, double* jpose, double* ji, double* nw, double* cost,
                                   int8_t* valid) {
    auto* o = static_cast<Oracle*>(h);
    for (size_t t = 0; t < o->nt(); ++t)
        for (int64_t k = o->offs[t]; k < o->offs[t + 1]; ++k) {
            const Obs& ob = o->obs[k];
            valid[k] = 0;
            if (!obsUsable(ob, o->state.cams.size())) continue;
            const Camera cam = effectiveCamera(*o, o->state, ob.cam);
            Lin L;
            if (!linearize(cam, activeIntrinsics(*o, ob.cam), o->state.points[t].data(), ob, o->opt.robust_loss,
                           o->opt.robust_loss_scale, o->refParam(), &L))
                continue;
            valid[k] = 1;
            std::memcpy(res + 2 * k, L.r, sizeof(L.r));
            std::memcpy(jp + 6 * k, L.Jp, sizeof(L.Jp));
            const Terms tm = primaryTerms(*o, o->state, ob.cam, L);
            std::fill(jpose + 2 * kP * k, jpose + 2 * kP * (k + 1), 0.0);
            if (o->active.cameraBlock[ob.cam] >= 0) std::memcpy(jpose + 2 * kP * k, tm.J[0], sizeof(tm.J[0]));
            std::memcpy(ji + 2 * kP * k, L.Ji, sizeof(L.Ji));
            nw[k] = L.nw;
            cost[k] = L.cost;
        }
    return 0;
}

int32_t orc_build(void* h, double damping, double* cost, int32_t* singular) {
    auto* o = static_cast<Oracle*>(h);
    try {
        bool s = false;
        build(*o, damping, cost, &s);
        *singular = s;
        return 0;
    } catch (const std::exception&) {
        return NumericalFailure;
    }
}

int32_t orc_pairs(void* h, int32_t* pairs) {
    auto* o = static_cast<Oracle*>(h);
    for (size_t s = 0; s < o->pairs.size(); ++s) {
        pairs[2 * s] = o->pairs[s].row;
        pairs[2 * s + 1] = o->pairs[s].col;
    }
    return 0;
}

int32_t orc_reduced(void* h, double* diag, double* off, double* grad, double* direct) {
    auto* o = static_cast<Oracle*>(h);
    std::copy(o->diag.begin(), o->diag.end(), diag);
    std::copy(o->off.begin(), o->off.end(), off);
    std::copy(o->gradient.begin(), o->gradient.end(), grad);
    std::copy(o->directRhs.begin(), o->directRhs.end(), direct);
    return 0;
}

int32_t orc_solve_linear(void* h, double* step, int32_t* converged, int32_t* iterations) {
    auto* o = static_cast<Oracle*>(h);
    try {
        std::vector<double> x;
        bool cv = false;
        int it = 0;
        solveLinear(*o, x, &cv, &it);
        std::copy(x.begin(), x.end(), step);
        *converged = cv;
        *iterations = it;
        return 0;
    } catch (const std::exception&) {
        return NumericalFailure;
    }
}

int32_t orc_back_substitute(void* h, const double* step, double* elim, double* dd, int32_t* success) {
    auto* o = static_cast<Oracle*>(h);
    std::vector<double> ps(step, step + static_cast<size_t>(o->active.primaryBlockCount) * kP), es;
    bool ok = false;
    backSubstitute(*o, ps, es, dd, &ok);
    std::copy(es.begin(), es.end(), elim);
    *success = ok;
    return 0;
}

double orc_cost(void* h) {
    auto* o = static_cast<Oracle*>(h);
    return objective(*o, o->state);
}

int32_t orc_general_build(void* h, double* cost, int32_t* counts) {
    auto* o = static_cast<Oracle*>(h);
    try {
        const int T = std::max(1, std::min<int>(o->threads, static_cast<int>(o->nt())));
        trackBoundaries(*o, T);
        if (!o->general) o->general = std::make_shared<GeneralEquations>();
        *cost = buildGeneral(*o, *o->general);
        counts[0] = o->general->P;
        counts[1] = o->general->E;
        counts[2] = static_cast<int32_t>(o->general->cpl.size());
        return 0;
    } catch (const std::exception&) {
        return NumericalFailure;
    }
}

int32_t orc_general_export(void* h, double* primary_matrix, double* gp, double* hee, double* ge, int32_t* cpl_index,
                           double* cpl) {
    auto* o = static_cast<Oracle*>(h);
    if (!o->general) return InvalidInput;
    const GeneralEquations& q = *o->general;
    const size_t n = static_cast<size_t>(q.P) * kP;
    std::fill(primary_matrix, primary_matrix + n * n, 0.0);
    for (int b = 0; b < q.P; ++b)
        for (int i = 0; i < kP; ++i)
            for (int j = 0; j < kP; ++j)
                primary_matrix[(static_cast<size_t>(b) * kP + i) * n + static_cast<size_t>(b) * kP + j] =
                    q.diag[static_cast<size_t>(b) * kP * kP + i * kP + j];
    for (const auto& kv : q.off) {
        const size_t r0 = static_cast<size_t>(kv.first.first) * kP, c0 = static_cast<size_t>(kv.first.second) * kP;
        for (int i = 0; i < kP; ++i)
            for (int j = 0; j < kP; ++j) {
                primary_matrix[(r0 + i) * n + c0 + j] = kv.second[i * kP + j];
                primary_matrix[(c0 + j) * n + r0 + i] = kv.second[i * kP + j];
            }
    }
    std::copy(q.gp.begin(), q.gp.end(), gp);
    std::copy(q.hee.begin(), q.hee.end(), hee);
    std::copy(q.ge.begin(), q.ge.end(), ge);
    size_t k = 0;
    for (const auto& kv : q.cpl) {
        cpl_index[2 * k] = kv.first.first;
        cpl_index[2 * k + 1] = kv.first.second;
        std::copy(kv.second.begin(), kv.second.end(), cpl + k * kP * kE);
        ++k;
    }
    return 0;
}

int32_t orc_general_solve(void* h, double damping, double tolerance, double* primary, double* eliminated,
                          int32_t* converged) {
    auto* o = static_cast<Oracle*>(h);
    if (!o->general) return InvalidInput;
    try {
        std::vector<double> x, y;
        bool cv = false;
        solveGeneralDamped(*o->general, damping, tolerance, o->opt.residual_gate != 0, x, y, &cv);
        std::copy(x.begin(), x.end(), primary);
        std::copy(y.begin(), y.end(), eliminated);
        *converged = cv;
        return 0;
    } catch (const std::exception&) {
        return NumericalFailure;
    }
}

// optimizePointsWithPlaMatrix, online reduced-Schur branch (BundleAdjustPlaMatrix.cpp:162-631),
// followed by finalizeBundleAdjustResult (BundleAdjustQuality.cpp:403-502).
int32_t orc_solve(void* h, orc_report* rep, double* camsOut, double* ptsOut, int8_t* validOut, double* rmsBefore,
                  double* rmsAfter, double* intrOut) {
    auto* o = static_cast<Oracle*>(h);
    std::memset(rep, 0, sizeof(*rep));
    const auto t0 = std::chrono::steady_clock::now();
    const Active& a = o->active;
    rep->active_tracks = a.activeTrackCount;
    rep->observation_count = a.observationCount;
    rep->rejected_initial_tracks = a.rejectedInitialTracks;
    o->state.cams = o->inputCams;
    o->state.points = o->initialPoints;
    initGroups(*o);
    if (a.observationCount == 0) {
        rep->status = InvalidInput;
        return rep->status;
    }
    double current = std::numeric_limits<double>::quiet_NaN(), damping = 0.0;
    int iterations = 0;
    bool converged = a.primaryBlockCount == 0 && a.trackBlockCount == 0;
    bool failed = false;
    std::vector<double> ps, es;
    if (o->opt.general_path) {
        solveGeneralPath(o, rep, &current, &iterations, &converged, &failed);
    } else
    try {
        if (converged) {
            current = objective(*o, o->state);
            rep->initial_cost = current;
            ++rep->objective_evaluations;
        }
        const int budget = std::max(1, o->opt.max_iterations);
        bool terminate = false;
        while (iterations < budget && !converged && !terminate) {
            bool relinearize = false;
            while (iterations < budget && !converged && !relinearize) {
                double cost = 0.0;
                bool singular = false;
                const auto ta = std::chrono::steady_clock::now();
                build(*o, damping, &cost, &singular);
                rep->assembly_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count();
                ++rep->linearizations;
                ++rep->objective_evaluations;
                current = cost;
                if (rep->linearizations == 1) rep->initial_cost = current;
                if (singular) {
                    ++iterations;
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                bool lconv = false;
                int lit = 0;
                const auto tl = std::chrono::steady_clock::now();
                try {
                    solveLinear(*o, ps, &lconv, &lit);
                } catch (const LinearFailure&) {
                    ++iterations;
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                rep->linear_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - tl).count();
                rep->linear_iterations += lit;
                ++iterations;
                if (!lconv) {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                double dd = 0.0;
                bool ok = false;
                backSubstitute(*o, ps, es, &dd, &ok);
                if (!ok || !std::isfinite(dd)) {
                    ++rep->rejected_steps;
                    damping = damping == 0.0 ? 1e-3 : damping * 10.0;
                    continue;
                }
                double rg = 0.0, rp = 0.0;
                stepRms(*o, ps, es, &rg, &rp);
                double cand = kInf, alpha = 1.0;
                bool accepted = false;
                State cs;
                for (int ls = 0; ls < o->opt.line_search_steps; ++ls) {
                    cs = applyStep(*o, o->state, ps, es, alpha);
                    cand = objective(*o, cs);
                    ++rep->objective_evaluations;
                    const double limit = current - o->opt.armijo_coefficient * alpha * dd;
                    if (std::isfinite(cand) && cand <= limit && cand < current) {
                        accepted = true;
                        break;
                    }
                    alpha *= 0.5;
                }
                if (std::getenv("PB_GPU_TRACE"))
                    std::fprintf(stderr,
                                 "ORACLE_TRACE it=%d cost=%.15e lambda=%.3e lin_it=%d dd=%.6e rms_global=%.3e "
                                 "rms_point=%.3e alpha=%.6g cand=%.15e accepted=%d\n",
                                 iterations, current, damping, lit, dd, rg, rp, alpha, cand, accepted ? 1 : 0);
                if (std::isfinite(cand) && cand < current && accepted) {
                    o->state = std::move(cs);
                    current = cand;
                    ++rep->accepted_steps;
                    damping /= 10.0;
                    converged = alpha * rg <= 1e-6 && alpha * rp <= 1e-6;
                    relinearize = !converged;
                } else {
                    ++rep->rejected_steps;
                    terminate = true;
                    relinearize = true;
                }
            }
        }
    } catch (const std::exception&) {
        failed = true;
    }
    rep->iterations = iterations;
    rep->final_cost = current;
    rep->solve_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (failed) {
        rep->status = NumericalFailure;
        return rep->status;
    }
    rep->status = converged ? Success : NoConvergence;
    rep->solution_usable = std::isfinite(current);
    const std::vector<Camera> refined = publishCameras(*o, o->state);
    for (size_t c = 0; c < refined.size(); ++c) storeCamera(refined[c], camsOut + c * ORC_CAMERA_STRIDE);
    for (size_t t = 0; t < o->nt(); ++t)
        for (int ax = 0; ax < 3; ++ax) ptsOut[t * 3 + ax] = o->state.points[t][ax];
    for (size_t g = 0; g < o->state.groups.size(); ++g)
        for (int p = 0; p < kP; ++p) intrOut[g * kP + p] = o->state.groups[g].params[p];
    // finalizeBundleAdjustResult
    std::vector<double> candidate;
    std::vector<char> valid(o->nt(), 0);
    for (size_t t = 0; t < o->nt(); ++t) {
        rmsBefore[t] = strictTrackRms(*o, o->inputCams, t, o->initialPoints[t].data());
        valid[t] = a.activeTrack[t] != 0;
        if (!valid[t]) {
            rmsAfter[t] = kInf;
            continue;
        }
        rmsAfter[t] = strictTrackRms(*o, refined, t, o->state.points[t].data());
        valid[t] = std::isfinite(rmsAfter[t]);
        if (valid[t]) candidate.push_back(rmsAfter[t]);
    }
    double threshold = kInf;
    if (o->opt.enable_point_filter) {
        threshold = std::isfinite(o->opt.filter_max_reproj_error) && o->opt.filter_max_reproj_error >= 0
                        ? o->opt.filter_max_reproj_error
                        : 0.0;
        std::vector<double> fin;
        for (double v : candidate)
            if (std::isfinite(v) && v >= 0.0) fin.push_back(v);
        if (!fin.empty() && std::isfinite(o->opt.filter_sigma_factor) && o->opt.filter_sigma_factor > 0.0)
            threshold = std::max(threshold, o->opt.filter_sigma_factor * finiteMedian(fin, 0.0));
    }
    rep->filter_threshold = threshold;
    double sb = 0.0, sa = 0.0;
    int opt = 0;
    for (size_t t = 0; t < o->nt(); ++t) {
        if (valid[t] && rmsAfter[t] > threshold) valid[t] = 0;
        if (valid[t]) {
            ++opt;
            sb += rmsBefore[t];
            sa += rmsAfter[t];
        }
        validOut[t] = valid[t];
    }
    rep->optimized_tracks = opt;
    rep->mean_rms_before = opt ? sb / opt : kInf;
    rep->mean_rms_after = opt ? sa / opt : kInf;
    rep->valid_track_ratio = o->nt() ? static_cast<double>(opt) / o->nt() : 0.0;
    if (opt == 0 && (rep->status == Success || rep->status == NoConvergence)) {
        rep->status = NumericalFailure;
        rep->solution_usable = 0;
    }
    return rep->status;
}

}  // extern "C"

// =================================================================================================
// Implicit-differentiation reference (adjoint of the converged fixed point).
//
// Not a restatement of reference code (the reference has no adjoint): it is the independent CPU
// check of the GPU backward pass.  Every observation's robust cost is written once more as a
// function of local chart variables around a fixed state (the solver's own retractions:
// rotation increment C2W' = D E(w)^T D C2W with E = Rx Ry Rz, world-frame centre increment or
// the 2-DoF gauge tangent on the sphere |C - C_anchor| = baseline, point increment X + s(X) dX,
// additive group intrinsics) and differentiated twice with hyper-dual numbers, which give exact
// first and second derivatives (no truncation error).  The Python side assembles the sparse
// Hessian from the per-observation blocks and solves it with a sparse direct factorisation.
// =================================================================================================
namespace orc {

// Hyper-dual number v + a e1 + b e2 + ab e1 e2 (e1^2 = e2^2 = 0).
struct HD {
    double v = 0.0, a = 0.0, b = 0.0, ab = 0.0;
    HD() = default;
    HD(double x) : v(x) {}  // NOLINT: constants promote implicitly
    HD(double x, double da, double db, double dab) : v(x), a(da), b(db), ab(dab) {}
};
inline HD operator+(const HD& x, const HD& y) { return {x.v + y.v, x.a + y.a, x.b + y.b, x.ab + y.ab}; }
inline HD operator-(const HD& x, const HD& y) { return {x.v - y.v, x.a - y.a, x.b - y.b, x.ab - y.ab}; }
inline HD operator-(const HD& x) { return {-x.v, -x.a, -x.b, -x.ab}; }
inline HD operator*(const HD& x, const HD& y) {
    return {x.v * y.v, x.v * y.a + x.a * y.v, x.v * y.b + x.b * y.v,
            x.v * y.ab + x.a * y.b + x.b * y.a + x.ab * y.v};
}
// f(x) for a scalar function with value f0, first derivative f1 and second derivative f2 at x.v
inline HD chain(const HD& x, double f0, double f1, double f2) {
    return {f0, f1 * x.a, f1 * x.b, f1 * x.ab + f2 * x.a * x.b};
}
inline HD recip(const HD& x) {
    const double i = 1.0 / x.v;
    return chain(x, i, -i * i, 2.0 * i * i * i);
}
inline HD operator/(const HD& x, const HD& y) { return x * recip(y); }
inline HD sqrt(const HD& x) {
    const double s = std::sqrt(x.v);
    return chain(x, s, 0.5 / s, -0.25 / (s * x.v));
}
inline HD sin(const HD& x) { return chain(x, std::sin(x.v), std::cos(x.v), -std::sin(x.v)); }
inline HD cos(const HD& x) { return chain(x, std::cos(x.v), -std::sin(x.v), -std::cos(x.v)); }
inline HD exp(const HD& x) {
    const double e = std::exp(x.v);
    return chain(x, e, e, e);
}
inline HD log1p(const HD& x) {
    const double i = 1.0 / (1.0 + x.v);
    return chain(x, std::log1p(x.v), i, -i * i);
}
inline double value(const HD& x) { return x.v; }
inline double value(double x) { return x; }

constexpr int kAdjMaxVars = 24;

// Fixed data of one observation's chart and the positions of its variables in the local vector.
struct ObsChart {
    double R[9], C[3];           // camera state (camera-to-world rotation, centre)
    double src[9];               // state intrinsics fx, fy, cx, cy, k1, k2, k3, p1, p2
    double refcx, refcy, su, sv;
    bool flip;
    bool tangent;                // gauge scale camera: centre on the sphere around the anchor
    double anchorC[3], e[3], Bw[6], baseline;
    double X[3], s;              // point and its step scale (s = 1 for a fixed track)
    double G[kP];                // group parameters (when the camera has a group)
    bool en[kP];
    double u, v, w;
    int loss;
    double scale;
    // local variable positions (-1: absent)
    int iw = -1, ic = -1, it = -1, ib = -1, ia = -1, ip = -1, iu = -1;
    int ik[kP];
};

template <class S>
S chartCost(const ObsChart& q, const S* z) {
    // rotation: C2W' = T C2W, T[r][c] = sg[r] E[c][r] sg[c], E = Rx(w0) Ry(w1) Rz(w2)
    const S w0 = z[q.iw], w1 = z[q.iw + 1], w2 = z[q.iw + 2];
    const S sx = sin(w0), cx = cos(w0), sy = sin(w1), cy = cos(w1), sz = sin(w2), cz = cos(w2);
    const S E[9] = {cy * cz, -(cy * sz), sy,
                    sx * sy * cz + cx * sz, cx * cz - sx * sy * sz, -(sx * cy),
                    sx * sz - cx * sy * cz, cx * sy * sz + sx * cz, cx * cy};
    const double sg[3] = {1.0, -1.0, -1.0};
    S Rn[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            S acc(0.0);
            for (int k = 0; k < 3; ++k) acc = acc + (sg[r] * sg[k]) * E[k * 3 + r] * q.R[k * 3 + c];
            Rn[r * 3 + c] = acc;
        }
    S Cn[3];
    if (q.tangent) {
        S dir[3];
        for (int i = 0; i < 3; ++i) dir[i] = q.e[i] + q.Bw[i] * z[q.it] + q.Bw[3 + i] * z[q.it + 1];
        const S len = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        const S bl = q.baseline + z[q.ib];
        for (int i = 0; i < 3; ++i) Cn[i] = q.anchorC[i] + z[q.ia + i] + bl * dir[i] / len;
    } else {
        for (int i = 0; i < 3; ++i) Cn[i] = q.C[i] + z[q.ic + i];
    }
    S d[3];
    for (int i = 0; i < 3; ++i) d[i] = (q.X[i] + (q.ip >= 0 ? q.s * z[q.ip + i] : S(0.0))) - Cn[i];
    const S xc = Rn[0] * d[0] + Rn[3] * d[1] + Rn[6] * d[2];
    const S yc = Rn[1] * d[0] + Rn[4] * d[1] + Rn[7] * d[2];
    const S zc = Rn[2] * d[0] + Rn[5] * d[1] + Rn[8] * d[2];
    const double fwd = q.flip ? -value(zc) : value(zc);
    if (!(fwd > 1e-9)) throw InvalidProjection("behind the camera");
    const S x = xc / zc, y = yc / zc;
    auto par = [&](int p, double base) -> S { return q.ik[p] >= 0 ? S(base) + z[q.ik[p]] : S(base); };
    const S fx = q.en[0] ? par(0, q.G[0]) : S(q.src[0]);
    const S aspect = q.en[1] ? exp(par(1, q.G[1])) : S(q.src[0] > 1e-12 ? q.src[1] / q.src[0] : 1.0);
    const S fy = fx * aspect;
    const S ccx = q.en[2] ? par(2, q.G[2]) + q.refcx : S(q.src[2]);
    const S ccy = q.en[3] ? par(3, q.G[3]) + q.refcy : S(q.src[3]);
    S dist[5];
    for (int p = 4; p < 9; ++p) dist[p - 4] = q.en[p] ? par(p, q.G[p]) : S(q.src[p]);
    const S r2 = x * x + y * y;
    const S radial = 1.0 + dist[0] * r2 + dist[1] * r2 * r2 + dist[2] * r2 * r2 * r2;
    const S xy2 = 2.0 * x * y;
    const S xd = x * radial + dist[3] * xy2 + dist[4] * (r2 + 2.0 * x * x);
    const S yd = y * radial + dist[3] * (r2 + 2.0 * y * y) + dist[4] * xy2;
    const S px = q.su * fx * xd + ccx, py = q.sv * fy * yd + ccy;
    const S r0 = px - (q.iu >= 0 ? q.u + z[q.iu] : S(q.u));
    const S r1 = py - (q.iu >= 0 ? q.v + z[q.iu + 1] : S(q.v));
    const S sq = q.w * (r0 * r0 + r1 * r1);
    if (!std::isfinite(value(sq)) || value(sq) < 0.0) throw InvalidProjection("non-finite residual");
    if (q.loss == 0) return 0.5 * sq;
    const double c2 = q.scale * q.scale;
    if (q.loss == 1) return value(sq) <= c2 ? 0.5 * sq : q.scale * sqrt(sq) - 0.5 * c2;
    return 0.5 * c2 * log1p(sq / c2);
}

}  // namespace orc

extern "C" {

// Replaces the state (cameras as published records, points, group parameters) so that the
// adjoint is evaluated where another solver stopped.
int32_t orc_set_state(void* h, const double* cams, const double* pts, const double* groups) {
    using namespace orc;
    auto* o = static_cast<Oracle*>(h);
    for (size_t c = 0; c < o->state.cams.size(); ++c) o->state.cams[c] = loadCamera(cams + c * ORC_CAMERA_STRIDE);
    for (size_t t = 0; t < o->nt(); ++t)
        for (int a = 0; a < 3; ++a) o->state.points[t][a] = pts[t * 3 + a];
    if (groups)
        for (size_t g = 0; g < o->state.groups.size(); ++g)
            for (int p = 0; p < kP; ++p) o->state.groups[g].params[p] = groups[g * kP + p];
    return 0;
}

// Variable numbering of the adjoint: camera c -> [6c, 6c + 6) (rotation increment, centre
// increment; the gauge scale camera's tangent coordinates in slots 3 and 4), track t ->
// 6 nc + 3 t, group g parameter p -> 6 nc + 3 nt + kP g + p, the gauge baseline -> 6 nc + 3 nt +
// kP ng, observation k (u, v) -> that + 1 + 2 k.  kind[id]: 0 unused, 1 solved for (free), 2 a
// parameter of the problem (fixed cameras and tracks, the baseline, the observations).
// geom (17 doubles): anchor, scale, baseline, e = C_scale - C_anchor (3), world tangent basis (6),
// anchor centre (3), 0.
int32_t orc_adjoint_layout(void* h, int64_t* n_vars, int8_t* kind, double* geom) {
    using namespace orc;
    auto* o = static_cast<Oracle*>(h);
    if (!o->refParam()) return 2;  // the adjoint charts are those of image-only problems
    const int64_t nc = static_cast<int64_t>(o->state.cams.size()), nt = static_cast<int64_t>(o->nt());
    const int64_t ng = static_cast<int64_t>(o->state.groups.size()), no = static_cast<int64_t>(o->obs.size());
    const int64_t base_g = 6 * nc + 3 * nt, id_b = base_g + kP * ng, base_o = id_b + 1;
    *n_vars = base_o + 2 * no;
    if (!kind) return 0;
    std::fill(kind, kind + *n_vars, 0);
    const Active& a = o->active;
    std::vector<char> camUsed(nc, 0);
    for (size_t t = 0; t < o->nt(); ++t) {
        if (!a.activeTrack[t]) continue;
        bool any = false;
        for (int64_t k = o->offs[t]; k < o->offs[t + 1]; ++k) {
            if (!obsUsable(o->obs[k], nc)) continue;
            any = true;
            camUsed[o->obs[k].cam] = 1;
            kind[base_o + 2 * k] = kind[base_o + 2 * k + 1] = 2;
        }
        if (any)
            for (int ax = 0; ax < 3; ++ax) kind[6 * nc + 3 * t + ax] = a.trackBlock[t] >= 0 ? 1 : 2;
    }
    for (int64_t c = 0; c < nc; ++c) {
        if (!camUsed[c]) continue;
        const bool free = a.cameraBlock[c] >= 0;
        const bool tangent = free && usesGaugeTangent(*o, c);
        for (int k = 0; k < 6; ++k) kind[6 * c + k] = free ? 1 : 2;
        if (tangent) kind[6 * c + 5] = 0;
    }
    for (int64_t g = 0; g < ng; ++g)
        for (int p = 0; p < kP; ++p)
            if (o->state.groups[g].enabled[p]) kind[base_g + kP * g + p] = 1;
    const bool gauge = o->gaugeScale >= 0 && a.cameraBlock[o->gaugeScale] >= 0 && usesGaugeTangent(*o, o->gaugeScale);
    if (gauge) {
        kind[id_b] = 2;
        for (int k = 0; k < 6; ++k) kind[6 * o->gaugeAnchor + k] = 2;
    }
    if (geom) {
        std::fill(geom, geom + 17, 0.0);
        geom[0] = o->gaugeAnchor;
        geom[1] = gauge ? o->gaugeScale : -1;
        geom[2] = o->gaugeBaseline;
        if (gauge) {
            const auto& A = o->state.cams[o->gaugeAnchor].C;
            const auto& Sc = o->state.cams[o->gaugeScale].C;
            const auto basis = gaugeBasis(*o, o->state);
            for (int i = 0; i < 3; ++i) geom[3 + i] = Sc[i] - A[i];
            for (int p = 0; p < 2; ++p) {
                const auto wb = targetCoords(basis[p].data());
                for (int i = 0; i < 3; ++i) geom[6 + 3 * p + i] = wb[i];
            }
            for (int i = 0; i < 3; ++i) geom[12 + i] = A[i];
        }
    }
    return 0;
}

// Per usable observation of an active track (in observation order, `count` of them): its local
// variables' global ids (kAdjMaxVars, -1 padded), robust cost, gradient and Hessian (row-major
// kAdjMaxVars^2) at state (+) z0, where z0 holds chart coordinates for every variable (NULL: 0).
// prior (3 * ng * kP): Hessian invSigma^2, gradient and cost of the group-intrinsic priors
// 0.5 (invSigma (theta - prior))^2 at the same state.  Returns 0, or 1 when an observation does
// not project.
int32_t orc_adjoint_local(void* h, const double* z0, int64_t* count, int32_t* ids, double* val, double* grad,
                          double* hess, double* prior) {
    using namespace orc;
    auto* o = static_cast<Oracle*>(h);
    if (!o->refParam()) return 2;  // the adjoint charts are those of image-only problems
    const int64_t nc = static_cast<int64_t>(o->state.cams.size()), nt = static_cast<int64_t>(o->nt());
    const int64_t ng = static_cast<int64_t>(o->state.groups.size());
    const int64_t base_g = 6 * nc + 3 * nt, id_b = base_g + kP * ng, base_o = id_b + 1;
    const Active& a = o->active;
    std::vector<int64_t> list;
    for (size_t t = 0; t < o->nt(); ++t) {
        if (!a.activeTrack[t]) continue;
        for (int64_t k = o->offs[t]; k < o->offs[t + 1]; ++k)
            if (obsUsable(o->obs[k], nc)) list.push_back(k);
    }
    *count = static_cast<int64_t>(list.size());
    if (prior)
        for (int64_t g = 0; g < ng; ++g)
            for (int p = 0; p < kP; ++p) {
                const Group& G = o->state.groups[g];
                const double w2 = G.enabled[p] ? G.invSigma[p] * G.invSigma[p] : 0.0;
                const double d = G.params[p] + (z0 ? z0[base_g + kP * g + p] : 0.0) - G.prior[p];
                prior[g * kP + p] = w2;                        // Hessian
                prior[(ng + g) * kP + p] = w2 * d;             // gradient
                prior[(2 * ng + g) * kP + p] = 0.5 * w2 * d * d;  // cost
            }
    if (!ids) return 0;
    std::vector<int64_t> trackOf(o->obs.size(), -1);
    for (size_t t = 0; t < o->nt(); ++t)
        for (int64_t k = o->offs[t]; k < o->offs[t + 1]; ++k) trackOf[k] = static_cast<int64_t>(t);
    const bool gauge = o->gaugeScale >= 0 && a.cameraBlock[o->gaugeScale] >= 0 && usesGaugeTangent(*o, o->gaugeScale);
    std::array<std::array<double, 3>, 2> basis{};
    if (gauge) basis = gaugeBasis(*o, o->state);
    const auto& refs = o->refCams.empty() ? o->inputCams : o->refCams;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) num_threads(o->threads)
    for (int64_t li = 0; li < static_cast<int64_t>(list.size()); ++li) {
        const int64_t k = list[li];
        const Obs& ob = o->obs[k];
        const int64_t t = trackOf[k];
        const int c = ob.cam;
        const Camera& cam = o->state.cams[c];
        ObsChart q{};
        std::memcpy(q.R, cam.R, sizeof q.R);
        std::memcpy(q.C, cam.C, sizeof q.C);
        const double src[9] = {cam.fx, cam.fy, cam.cx, cam.cy, cam.k1, cam.k2, cam.k3, cam.p1, cam.p2};
        std::memcpy(q.src, src, sizeof src);
        q.refcx = refs[c].cx;
        q.refcy = refs[c].cy;
        q.su = cam.su;
        q.sv = cam.sv;
        q.flip = cam.flip;
        q.tangent = gauge && c == o->gaugeScale;
        int64_t gid[kAdjMaxVars];
        int m = 0;
        q.iw = m;
        for (int i = 0; i < 3; ++i) gid[m++] = 6 * c + i;
        if (q.tangent) {
            const auto& A = o->state.cams[o->gaugeAnchor].C;
            for (int i = 0; i < 3; ++i) {
                q.anchorC[i] = A[i];
                q.e[i] = cam.C[i] - A[i];
            }
            for (int p = 0; p < 2; ++p) {
                const auto wb = targetCoords(basis[p].data());
                for (int i = 0; i < 3; ++i) q.Bw[3 * p + i] = wb[i];
            }
            q.baseline = o->gaugeBaseline;
            q.it = m;
            gid[m++] = 6 * c + 3;
            gid[m++] = 6 * c + 4;
            q.ib = m;
            gid[m++] = id_b;
            q.ia = m;
            for (int i = 0; i < 3; ++i) gid[m++] = 6 * o->gaugeAnchor + 3 + i;
        } else {
            q.ic = m;
            for (int i = 0; i < 3; ++i) gid[m++] = 6 * c + 3 + i;
        }
        for (int i = 0; i < 3; ++i) q.X[i] = o->state.points[t][i];
        q.s = a.trackBlock[t] >= 0 ? referencePointScale(q.X) : 1.0;
        q.ip = m;
        for (int i = 0; i < 3; ++i) gid[m++] = 6 * nc + 3 * t + i;
        for (int p = 0; p < kP; ++p) q.ik[p] = -1;
        const int g = o->state.groups.empty() ? -1 : a.calibGroupByCamera[c];
        if (g >= 0) {
            const Group& G = o->state.groups[g];
            for (int p = 0; p < kP; ++p) {
                q.G[p] = G.params[p];
                q.en[p] = G.enabled[p];
                if (G.enabled[p]) {
                    q.ik[p] = m;
                    gid[m++] = base_g + kP * g + p;
                }
            }
        }
        q.iu = m;
        gid[m++] = base_o + 2 * k;
        gid[m++] = base_o + 2 * k + 1;
        const double ms = sanitizedScale(ob);
        q.u = ob.u;
        q.v = ob.v;
        q.w = sanitizedWeight(ob) / (ms * ms);
        q.loss = o->opt.robust_loss;
        q.scale = o->opt.robust_loss_scale;
        int32_t* oid = ids + li * kAdjMaxVars;
        double* og = grad + li * kAdjMaxVars;
        double* oh = hess + li * kAdjMaxVars * kAdjMaxVars;
        for (int i = 0; i < kAdjMaxVars; ++i) {
            oid[i] = i < m ? static_cast<int32_t>(gid[i]) : -1;
            og[i] = 0.0;
        }
        std::fill(oh, oh + kAdjMaxVars * kAdjMaxVars, 0.0);
        try {
            HD z[kAdjMaxVars];
            for (int i = 0; i < m; ++i) z[i] = HD(z0 ? z0[gid[i]] : 0.0);
            for (int i = 0; i < m; ++i)
                for (int j = i; j < m; ++j) {
                    z[i].a = 1.0;
                    z[j].b = 1.0;
                    const HD f = chartCost(q, z);
                    z[i].a = 0.0;
                    z[j].b = 0.0;
                    oh[i * kAdjMaxVars + j] = oh[j * kAdjMaxVars + i] = f.ab;
                    if (j == i) og[i] = f.a;
                    if (i == 0 && j == 0) val[li] = f.v;
                }
        } catch (const InvalidProjection&) {
#pragma omp atomic write
            bad = 1;
        }
    }
    return bad;
}

}  // extern "C"
