// svg.cu — SVG path data to path batches, on the host: lyon's PathParser
// (crates/extra/src/parser.rs:138-490) over many strings at once, writing the batch layout
// (verbs, points, offsets; include/lyon_gpu.h) that the tessellation kernels read, so a scene
// of path strings goes to the GPU without a per-path builder in between.
//
// Strings are parsed on all host threads in two passes (sizes, then output at scanned offsets).
// Arcs become quadratic béziers as lyon's SvgArc / Arc do (crates/geom/src/arc.rs:58-138,
// 668-703), in f32 (cos, sin and tan evaluated in f64 and rounded once, identically on host and
// device); `angle_from_x_axis` is euclid 0.22.9's fast_atan2,
// as lyon's. One detail differs from lyon and is stated where it applies: only ASCII digits count
// as numeric (lyon accepts any Unicode numeric character into a number, which then fails to
// parse).
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lyon_gpu.h"
#include "decimal.cuh"
#include "kernels.h"

#define HD __host__ __device__

namespace {

constexpr float PI_F = 3.14159265358979323846f;

struct Pt {
    float x, y;
};

// Source (parser.rs:51-120): the current character, line and column. UTF-8 input.
struct Source {
    const unsigned char* p;
    const unsigned char* end;
    uint32_t current = ' ';
    bool finished = false;
    int32_t line = 0, col = 0;

    HD bool next_char(uint32_t* c) {
        if (p >= end) return false;
        uint32_t b = *p++;
        int extra = b >= 0xF0 ? 3 : b >= 0xE0 ? 2 : b >= 0xC0 ? 1 : 0;
        uint32_t v = extra == 3 ? (b & 0x07) : extra == 2 ? (b & 0x0F) : extra == 1 ? (b & 0x1F) : b;
        for (int k = 0; k < extra && p < end; ++k) v = (v << 6) | (*p++ & 0x3F);
        *c = v;
        return true;
    }
    HD Source(const char* s, size_t n)
        : p(reinterpret_cast<const unsigned char*>(s)),
          end(reinterpret_cast<const unsigned char*>(s) + n) {
        uint32_t c;
        if (next_char(&c)) {
            current = c;
        } else {
            current = ' ';
            finished = true;
        }
        line = current == '\n' ? 1 : 0;
        col = 0;
    }
    // char::is_whitespace (the Unicode White_Space set) or ','.
    HD static bool is_ws(uint32_t c) {
        return (c >= 0x09 && c <= 0x0D) || c == 0x20 || c == 0x85 || c == 0xA0 || c == 0x1680 ||
               (c >= 0x2000 && c <= 0x200A) || c == 0x2028 || c == 0x2029 || c == 0x202F ||
               c == 0x205F || c == 0x3000;
    }
    HD void skip_whitespace() {
        while (!finished && (is_ws(current) || current == ',')) advance_one();
    }
    HD void advance_one() {
        if (finished) return;
        uint32_t c;
        if (!next_char(&c)) {
            current = '~';
            finished = true;
        } else if (c == '\n') {
            current = '\n';
            ++line;
            col = -1;
        } else {
            current = c;
            ++col;
        }
    }
};

// The output: lyon's Path builder (crates/path/src/path.rs:517-592, no validation in release
// builds), writing verbs and points (and the endpoint attribute, when parsed, into `widths`)
// or only counting them.
struct Out {
    uint8_t* verbs = nullptr;
    float* points = nullptr;
    float* widths = nullptr;
    uint64_t nv = 0, np = 0;
    Pt first{0.0f, 0.0f};
    float first_w = 0.0f;
    HD void point(Pt p, float w) {
        if (points) {
            points[2 * np] = p.x;
            points[2 * np + 1] = p.y;
        }
        if (widths) widths[np] = w;
        ++np;
    }
    HD void verb(uint8_t v) {
        if (verbs) verbs[nv] = v;
        ++nv;
    }
    HD void begin(Pt at, float w) {
        first = at;
        first_w = w;
        point(at, w);
        verb(LYON_VERB_BEGIN);
    }
    HD void line_to(Pt to, float w) {
        point(to, w);
        verb(LYON_VERB_LINE_TO);
    }
    HD void quad_to(Pt c, Pt to, float w) {
        point(c, 0.0f);
        point(to, w);
        verb(LYON_VERB_QUADRATIC_TO);
    }
    HD void cubic_to(Pt c1, Pt c2, Pt to, float w) {
        point(c1, 0.0f);
        point(c2, 0.0f);
        point(to, w);
        verb(LYON_VERB_CUBIC_TO);
    }
    HD void end(bool close) {
        if (close) point(first, first_w);
        verb(close ? LYON_VERB_CLOSE : LYON_VERB_END);
    }
};

// ---- arcs (crates/geom/src/arc.rs) -------------------------------------------------------

// lyon takes cos, sin and tan of f32 angles from the platform's f32 libm; host and device libms
// differ in the last bit, and an arc's segment count ceil(sweep / (pi / 4)) can turn on that
// bit. Both parsers evaluate them in f64 and round once (within an ulp of any f32 libm's).
HD float cos_r(float x) { return (float)cos((double)x); }
HD float sin_r(float x) { return (float)sin((double)x); }
HD float tan_r(float x) { return (float)tan((double)x); }

// Rotation2D::transform_point / transform_vector (euclid): the rotation matrix of `angle`.
HD Pt rotate(float angle, Pt v) {
    const float s = sin_r(angle), c = cos_r(angle);
    return Pt{v.x * c - v.y * s, v.x * s + v.y * c};
}

// euclid 0.22.9 `Vector2D::angle_from_x_axis` = `Trig::fast_atan2(y, x)` (euclid src/trig.rs):
// the published polynomial approximation of atan on [0, 1] (math.stackexchange.com question
// 1098487, answer 1105038), reflected into the octant of (x, y); f32, evaluated left to right.
HD float angle_from_x_axis(Pt v) {
    const float x_abs = fabsf(v.x), y_abs = fabsf(v.y);
    const float a = fminf(x_abs, y_abs) / fmaxf(x_abs, y_abs);
    const float s = a * a;
    float r = ((-0.0464964749f * s + 0.15931422f) * s - 0.327622764f) * s * a + a;
    if (y_abs > x_abs) r = 1.57079632679489661923f - r;
    if (v.x < 0.0f) r = PI_F - r;
    if (v.y < 0.0f) r = -r;
    return r;
}

struct Arc {
    Pt center, radii;
    float start_angle, sweep_angle, x_rotation;
};

// Arc::from_svg_arc (arc.rs:58-138).
HD Arc from_svg_arc(Pt from, Pt to, Pt radii, float x_rotation, bool large_arc, bool sweep) {
    float rx = fabsf(radii.x), ry = fabsf(radii.y);
    const float xr = fmodf(x_rotation, 2.0f * PI_F);
    const float cos_phi = cos_r(xr), sin_phi = sin_r(xr);
    const float hd_x = (from.x - to.x) / 2.0f, hd_y = (from.y - to.y) / 2.0f;
    const float hs_x = (from.x + to.x) / 2.0f, hs_y = (from.y + to.y) / 2.0f;
    const Pt p{cos_phi * hd_x + sin_phi * hd_y, -sin_phi * hd_x + cos_phi * hd_y};
    const float rf = p.x * p.x / (rx * rx) + p.y * p.y / (ry * ry);
    if (rf > 1.0f) {
        const float scale = sqrtf(rf);
        rx *= scale;
        ry *= scale;
    }
    const float rxry = rx * ry, rxpy = rx * p.y, rypx = ry * p.x;
    const float sum_of_sq = rxpy * rxpy + rypx * rypx;
    const float sign_coe = large_arc == sweep ? -1.0f : 1.0f;
    const float coe = sign_coe * sqrtf(fabsf((rxry * rxry - sum_of_sq) / sum_of_sq));
    const float tcx = coe * rxpy / ry;
    const float tcy = -coe * rypx / rx;
    const Pt center{cos_phi * tcx - sin_phi * tcy + hs_x, sin_phi * tcx + cos_phi * tcy + hs_y};
    const Pt start_v{(p.x - tcx) / rx, (p.y - tcy) / ry};
    const Pt end_v{(-p.x - tcx) / rx, (-p.y - tcy) / ry};
    const float two_pi = 2.0f * PI_F;
    const float start_angle = angle_from_x_axis(start_v);
    float sweep_angle = fmodf(angle_from_x_axis(end_v) - start_angle, two_pi);
    if (sweep && sweep_angle < 0.0f) {
        sweep_angle += two_pi;
    } else if (!sweep && sweep_angle > 0.0f) {
        sweep_angle -= two_pi;
    }
    return Arc{center, Pt{rx, ry}, start_angle, sweep_angle, x_rotation};
}

// f32::signum: 1 for +0 and positives, -1 for -0 and negatives, NaN for NaN.
HD float signum(float v) { return v != v ? v : ((lg::f32_bits(v) >> 31) ? -1.0f : 1.0f); }

// arc_to_quadratic_beziers_with_t (arc.rs:668-703); `cb(ctrl, to, t_end)`. Returns false where
// lyon's `cast::<S, i32>(n_steps).unwrap()` would panic (a NaN or huge step count).
template <class F>
HD bool arc_to_quadratics(const Arc& arc, F&& cb) {
    const float sign = signum(arc.sweep_angle);
    float sweep_angle = fabsf(arc.sweep_angle);
    if (!(sweep_angle <= PI_F * 2.0f)) sweep_angle = PI_F * 2.0f;  // f32::min (NaN: the other)
    const float n_steps = ceilf(sweep_angle / (PI_F / 4.0f));
    if (!(n_steps >= 0.0f && n_steps < 2147483648.0f)) return false;
    const float step = sweep_angle / n_steps * sign;
    float t0 = 0.0f;
    const float dt = 1.0f / n_steps;
    const float alpha = tan_r(step * 0.5f);
    const int n = (int)n_steps;
    for (int i = 0; i < n; ++i) {
        const float a1 = arc.start_angle + step * (float)i;
        const float a2 = arc.start_angle + step * (float)(i + 1);
        const Pt v1 = rotate(arc.x_rotation, Pt{arc.radii.x * cos_r(a1), arc.radii.y * sin_r(a1)});
        const Pt v2 = rotate(arc.x_rotation, Pt{arc.radii.x * cos_r(a2), arc.radii.y * sin_r(a2)});
        const Pt from{arc.center.x + v1.x, arc.center.y + v1.y};
        const Pt to{arc.center.x + v2.x, arc.center.y + v2.y};
        const Pt tan = rotate(arc.x_rotation, Pt{-arc.radii.x * sin_r(a1), arc.radii.y * cos_r(a1)});
        const Pt ctrl{from.x + tan.x * alpha, from.y + tan.y * alpha};
        const float t1 = i + 1 == n ? 1.0f : t0 + dt;
        cb(ctrl, to, t1);
        t0 = t1;
    }
    return true;
}

// ---- the parser (parser.rs:138-490) -----------------------------------------------------

struct Parser {
    uint32_t num_attributes;  // 0 or 1
    int64_t stop_at;          // code point, or -1
    Pt current{0.0f, 0.0f};
    float attr = 0.0f;        // the current endpoint's attribute
    bool need_end = false;
    int32_t err = LYON_OK, err_line = 0, err_col = 0;

    HD bool fail(int code, int32_t line, int32_t col) {
        err = code;
        err_line = line;
        err_col = col;
        return false;
    }

    // parse_number (parser.rs:413-467): [-]digits[.digits][(e|E)[-]digits], then Rust's
    // f32::from_str on that text (correctly rounded: decimal_to_f32).
    HD bool number(Source& s, float* out) {
        s.skip_whitespace();
        const int32_t line = s.line, col = s.col;
        lg::DecimalBuilder b;
        if (s.current == '-') {
            b.d.negative = true;
            s.advance_one();
        }
        size_t mant = 0;
        while (s.current >= '0' && s.current <= '9') {
            b.digit((int)(s.current - '0'));
            s.advance_one();
            ++mant;
        }
        if (s.current == '.') {
            b.point();
            s.advance_one();
            while (s.current >= '0' && s.current <= '9') {
                b.digit((int)(s.current - '0'));
                s.advance_one();
                ++mant;
            }
        }
        bool exp_ok = true;
        long long e = 0;
        if (s.current == 'e' || s.current == 'E') {
            s.advance_one();
            bool eneg = false;
            if (s.current == '-') {
                eneg = true;
                s.advance_one();
            }
            size_t ed = 0;
            while (s.current >= '0' && s.current <= '9') {
                if (e < 100000000) e = e * 10 + (long long)(s.current - '0');
                s.advance_one();
                ++ed;
            }
            if (eneg) e = -e;
            exp_ok = ed > 0;
        }
        if (mant == 0 || !exp_ok) return fail(LYON_SVG_ERR_NUMBER, line, col);
        *out = b.finish(e);
        return true;
    }

    HD bool flag(Source& s, bool* out) {  // parser.rs:469-490
        s.skip_whitespace();
        if (s.current == '1' || s.current == '0') {
            *out = s.current == '1';
            s.advance_one();
            return true;
        }
        return fail(LYON_SVG_ERR_FLAG, s.line, s.col);
    }

    HD bool attributes(Source& s) {  // parser.rs:384-395
        if (num_attributes == 0) return true;
        return number(s, &attr);
    }

    HD bool point(Source& s, bool rel, Pt* out) {  // parser.rs:397-411
        float x, y;
        if (!number(s, &x) || !number(s, &y)) return false;
        if (rel) {
            x += current.x;
            y += current.y;
        }
        *out = Pt{x, y};
        return true;
    }

    HD bool endpoint(Source& s, bool rel, Pt* out) {  // parser.rs:371-382
        if (!point(s, rel, out)) return false;
        current = *out;
        return attributes(s);
    }

    HD Pt smooth_ctrl(const Pt* prev) const {  // parser.rs:363-369
        if (!prev) return current;
        return Pt{current.x + (current.x - prev->x), current.y + (current.y - prev->y)};
    }

    // parse (parser.rs:154-175) with parse_path (177-361).
    HD void parse(Source& s, Out& o) {
        need_end = false;
        run(s, o);
        if (need_end) o.end(false);
    }

    HD void run(Source& s, Out& o) {
        current = Pt{0.0f, 0.0f};
        Pt first_position{0.0f, 0.0f};
        bool need_start = false;
        Pt prev_cubic{0, 0}, prev_quad{0, 0};
        bool has_cubic = false, has_quad = false;
        uint32_t implicit_cmd = 'M';
        s.skip_whitespace();
        while (!s.finished) {
            uint32_t cmd = s.current;
            const int32_t cmd_line = s.line, cmd_col = s.col;
            if (stop_at >= 0 && (int64_t)cmd == stop_at) break;
            const bool alpha = (cmd >= 'a' && cmd <= 'z') || (cmd >= 'A' && cmd <= 'Z');
            if (alpha) {
                s.advance_one();
            } else {
                cmd = implicit_cmd;
            }
            if (need_start && cmd != 'm' && cmd != 'M') {
                fail(LYON_SVG_ERR_MISSING_MOVE_TO, cmd_line, cmd_col);
                return;
            }
            const bool rel = cmd >= 'a' && cmd <= 'z';
            Pt to, c1, c2;
            switch (cmd) {
                case 'l':
                case 'L':
                    if (!endpoint(s, rel, &to)) return;
                    o.line_to(to, attr);
                    break;
                case 'h':
                case 'H': {
                    float x;
                    if (!number(s, &x)) return;
                    if (rel) x += current.x;
                    to = Pt{x, current.y};
                    current = to;
                    if (!attributes(s)) return;
                    o.line_to(to, attr);
                    break;
                }
                case 'v':
                case 'V': {
                    float y;
                    if (!number(s, &y)) return;
                    if (rel) y += current.y;
                    to = Pt{current.x, y};
                    current = to;
                    if (!attributes(s)) return;
                    o.line_to(to, attr);
                    break;
                }
                case 'q':
                case 'Q':
                    if (!point(s, rel, &c1) || !endpoint(s, rel, &to)) return;
                    prev_quad = c1;
                    has_quad = true;
                    o.quad_to(c1, to, attr);
                    break;
                case 't':
                case 'T':
                    c1 = smooth_ctrl(has_quad ? &prev_quad : nullptr);
                    if (!endpoint(s, rel, &to)) return;
                    prev_quad = c1;
                    has_quad = true;
                    o.quad_to(c1, to, attr);
                    break;
                case 'c':
                case 'C':
                    if (!point(s, rel, &c1) || !point(s, rel, &c2) || !endpoint(s, rel, &to))
                        return;
                    prev_cubic = c2;
                    has_cubic = true;
                    o.cubic_to(c1, c2, to, attr);
                    break;
                case 's':
                case 'S':
                    c1 = smooth_ctrl(has_cubic ? &prev_cubic : nullptr);
                    if (!point(s, rel, &c2) || !endpoint(s, rel, &to)) return;
                    prev_cubic = c2;
                    has_cubic = true;
                    o.cubic_to(c1, c2, to, attr);
                    break;
                case 'a':
                case 'A': {
                    const float prev_attr = attr;
                    const Pt from = current;
                    float rx, ry, xrot;
                    bool large_arc, sweep;
                    if (!number(s, &rx) || !number(s, &ry) || !number(s, &xrot) ||
                        !flag(s, &large_arc) || !flag(s, &sweep) || !endpoint(s, rel, &to))
                        return;
                    // SvgArc::is_straight_line (arc.rs:534-539)
                    const float eps = 1.1920929e-7f;  // f32::EPSILON
                    if (fabsf(rx) <= eps || fabsf(ry) <= eps || (from.x == to.x && from.y == to.y)) {
                        o.line_to(to, attr);
                    } else {
                        // Angle::degrees: x * (PI / 180) in f32.
                        const Arc arc = from_svg_arc(from, to, Pt{rx, ry}, xrot * (PI_F / 180.0f),
                                                     large_arc, sweep);
                        const float end_attr = attr;
                        const bool ok = arc_to_quadratics(arc, [&](Pt c, Pt t, float t1) {
                            const float w = prev_attr * (1.0f - t1) + end_attr * t1;
                            o.quad_to(c, t, w);
                        });
                        if (!ok) {
                            fail(LYON_ERR_INTERNAL, cmd_line, cmd_col);
                            return;
                        }
                    }
                    break;
                }
                case 'm':
                case 'M':
                    if (need_end) {
                        o.end(false);
                        need_end = false;
                    }
                    if (!endpoint(s, rel, &to)) return;
                    first_position = to;
                    o.begin(to, attr);
                    need_end = true;
                    need_start = false;
                    break;
                case 'z':
                case 'Z':
                    o.end(true);
                    current = first_position;
                    need_end = false;
                    need_start = true;
                    break;
                default:
                    fail(LYON_SVG_ERR_COMMAND, cmd_line, cmd_col);
                    return;
            }
            if (cmd == 'c' || cmd == 'C' || cmd == 's' || cmd == 'S') {
                has_quad = false;
            } else if (cmd == 'q' || cmd == 'Q' || cmd == 't' || cmd == 'T') {
                has_cubic = false;
            } else {
                has_cubic = has_quad = false;
            }
            implicit_cmd = cmd == 'm' ? 'l' : cmd == 'M' ? 'L' : cmd == 'z' ? 'm' : cmd == 'Z' ? 'M' : cmd;
            s.skip_whitespace();
        }
    }
};

// ---- on the device -----------------------------------------------------------------------

// One thread parses one string with the same Parser (lyon's PathParser), counting (write false:
// verb/point counts and the parse status) or writing at the scanned offsets.
__global__ void svg_parse_kernel(const char* text, const uint64_t* string_offsets, uint32_t n,
                                 uint32_t num_attributes, long long stop_at, int write,
                                 uint32_t* verb_counts, uint32_t* point_counts, int32_t* status,
                                 int32_t* error_line, int32_t* error_column,
                                 const uint64_t* verb_offsets, const uint64_t* point_offsets,
                                 uint8_t* verbs, float* points, float* widths) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        Source src(text + string_offsets[i], string_offsets[i + 1] - string_offsets[i]);
        Out o;
        if (write) {
            o.verbs = verbs + verb_offsets[i];
            o.points = points + 2 * point_offsets[i];
            o.widths = widths ? widths + point_offsets[i] : nullptr;
        }
        Parser p;
        p.num_attributes = num_attributes;
        p.stop_at = stop_at;
        p.parse(src, o);
        if (!write) {
            verb_counts[i] = (uint32_t)o.nv;
            point_counts[i] = (uint32_t)o.np;
            status[i] = p.err;
            error_line[i] = p.err_line;
            error_column[i] = p.err_col;
        }
    }
}

}  // namespace

namespace lg {
cudaError_t launch_svg_parse(const char* text, const uint64_t* string_offsets, uint32_t n,
                             uint32_t num_attributes, long long stop_at, bool write,
                             uint32_t* verb_counts, uint32_t* point_counts, int32_t* status,
                             int32_t* error_line, int32_t* error_column,
                             const uint64_t* verb_offsets, const uint64_t* point_offsets,
                             uint8_t* verbs, float* points, float* widths, int num_sms,
                             cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t threads = 128;
    uint32_t blocks = (n + threads - 1) / threads;
    const uint32_t cap = (uint32_t)(num_sms > 0 ? num_sms : 1) * 16u;
    if (blocks > cap) blocks = cap;
    svg_parse_kernel<<<blocks, threads, 0, stream>>>(
        text, string_offsets, n, num_attributes, stop_at, write ? 1 : 0, verb_counts,
        point_counts, status, error_line, error_column, verb_offsets, point_offsets, verbs,
        points, widths);
    note_launches(1);
    return cudaGetLastError();
}
}  // namespace lg



extern "C" int lyon_svg_parse_paths(const char* text, const uint64_t* string_offsets,
                                    uint32_t num_strings, const lyon_svg_parse_options* options,
                                    uint8_t* verbs, uint64_t verb_capacity, float* points,
                                    uint64_t point_capacity, float* widths,
                                    uint32_t* verb_offsets, uint32_t* point_offsets,
                                    int32_t* status, int32_t* error_line, int32_t* error_column,
                                    uint64_t* total_verbs, uint64_t* total_points) {
    if ((num_strings && (!text || !string_offsets)) || !total_verbs || !total_points)
        return LYON_ERR_INVALID_ARGUMENT;
    const uint32_t num_attributes = options ? options->num_attributes : 0;
    if (num_attributes > 1) return LYON_ERR_UNSUPPORTED;
    const int64_t stop_at = options ? options->stop_at : -1;
    uint32_t threads = options && options->num_threads ? options->num_threads
                                                       : std::thread::hardware_concurrency();
    if (threads == 0) threads = 1;
    if (threads > 256) threads = 256;
    std::vector<uint64_t> nv(num_strings + 1, 0), np(num_strings + 1, 0);
    std::vector<int32_t> st(num_strings, LYON_OK), el(num_strings, 0), ec(num_strings, 0);

    auto run = [&](bool write) {
        std::atomic<uint32_t> next{0};
        auto worker = [&]() {
            for (;;) {
                const uint32_t b = next.fetch_add(256);
                if (b >= num_strings) break;
                const uint32_t e = b + 256 < num_strings ? b + 256 : num_strings;
                for (uint32_t i = b; i < e; ++i) {
                    Source s(text + string_offsets[i], string_offsets[i + 1] - string_offsets[i]);
                    Out o;
                    if (write) {
                        o.verbs = verbs + nv[i];
                        o.points = points + 2 * np[i];
                        o.widths = widths ? widths + np[i] : nullptr;
                    }
                    Parser p;
                    p.num_attributes = num_attributes;
                    p.stop_at = stop_at;
                    p.parse(s, o);
                    if (!write) {
                        nv[i + 1] = o.nv;
                        np[i + 1] = o.np;
                        st[i] = p.err;
                        el[i] = p.err_line;
                        ec[i] = p.err_col;
                    }
                }
            }
        };
        const uint32_t t = threads < (num_strings + 255) / 256 ? threads : (num_strings + 255) / 256;
        std::vector<std::thread> pool;
        for (uint32_t k = 1; k < t; ++k) pool.emplace_back(worker);
        worker();
        for (auto& th : pool) th.join();
    };
    run(false);
    for (uint32_t i = 0; i < num_strings; ++i) {
        nv[i + 1] += nv[i];
        np[i + 1] += np[i];
    }
    *total_verbs = nv[num_strings];
    *total_points = np[num_strings];
    if (*total_verbs > 0xFFFFFFFFull || *total_points > 0xFFFFFFFFull) return LYON_ERR_UNSUPPORTED;
    if (status) memcpy(status, st.data(), num_strings * sizeof(int32_t));
    if (error_line) memcpy(error_line, el.data(), num_strings * sizeof(int32_t));
    if (error_column) memcpy(error_column, ec.data(), num_strings * sizeof(int32_t));
    if (!verbs || !points || !verb_offsets || !point_offsets || verb_capacity < *total_verbs ||
        point_capacity < *total_points)
        return LYON_ERR_CAPACITY;
    for (uint32_t i = 0; i <= num_strings; ++i) {
        verb_offsets[i] = (uint32_t)nv[i];
        point_offsets[i] = (uint32_t)np[i];
    }
    run(true);
    return LYON_OK;
}
