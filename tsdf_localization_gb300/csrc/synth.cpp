// Seeded synthetic workloads for the sensor update: worlds made of oriented
// boxes, their TSDF in the reference's raw cell format (int16 value in mm and
// int16 weight packed in a uint32, include/tsdf_localization/util/tsdf.h:11-33)
// stored as chunks of edge^3 cells, ray-cast LiDAR scans, scan reduction and
// particle clouds.  Host code (OpenMP); nothing here runs on the sensor-update
// path itself.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <omp.h>

namespace {

struct Rng {  // splitmix64: identical stream on every platform
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    double normal()
    {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

// Oriented box: centre c, rotation R (rows = local axes in world), half size h.
struct Box {
    double c[3];
    double R[3][3];
    double h[3];
    double lo[3], hi[3];  // world AABB
};

void rot_rpy(double r, double p, double y, double R[3][3])
{
    double cr = std::cos(r), sr = std::sin(r), cp = std::cos(p), sp = std::sin(p), cy = std::cos(y), sy = std::sin(y);
    // world = Rz(y) Ry(p) Rx(r) local; store rows of the inverse (= columns of the forward)
    double F[3][3] = {{cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr},
                      {sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr},
                      {-sp, cp * sr, cp * cr}};
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) R[a][b] = F[b][a];
}

Box make_box(double cx, double cy, double cz, double hx, double hy, double hz, double r = 0, double p = 0,
             double y = 0)
{
    Box b;
    b.c[0] = cx; b.c[1] = cy; b.c[2] = cz;
    b.h[0] = hx; b.h[1] = hy; b.h[2] = hz;
    rot_rpy(r, p, y, b.R);
    for (int a = 0; a < 3; ++a) {
        double e = 0;
        for (int k = 0; k < 3; ++k) e += std::fabs(b.R[k][a]) * b.h[k];
        b.lo[a] = b.c[a] - e;
        b.hi[a] = b.c[a] + e;
    }
    return b;
}

double box_sdf(const Box& b, const double p[3])
{
    double d[3], q[3];
    for (int a = 0; a < 3; ++a) d[a] = p[a] - b.c[a];
    for (int k = 0; k < 3; ++k) q[k] = std::fabs(b.R[k][0] * d[0] + b.R[k][1] * d[1] + b.R[k][2] * d[2]) - b.h[k];
    double ox = std::max(q[0], 0.0), oy = std::max(q[1], 0.0), oz = std::max(q[2], 0.0);
    double outside = std::sqrt(ox * ox + oy * oy + oz * oz);
    double inside = std::min(std::max(q[0], std::max(q[1], q[2])), 0.0);
    return outside + inside;
}

// Ray / box: returns entry distance or +inf.
double box_ray(const Box& b, const double o[3], const double dir[3])
{
    double lo = 0, hi = std::numeric_limits<double>::infinity();
    for (int k = 0; k < 3; ++k) {
        double oo = b.R[k][0] * (o[0] - b.c[0]) + b.R[k][1] * (o[1] - b.c[1]) + b.R[k][2] * (o[2] - b.c[2]);
        double dd = b.R[k][0] * dir[0] + b.R[k][1] * dir[1] + b.R[k][2] * dir[2];
        if (std::fabs(dd) < 1e-12) {
            if (oo < -b.h[k] || oo > b.h[k]) return std::numeric_limits<double>::infinity();
            continue;
        }
        double t1 = (-b.h[k] - oo) / dd, t2 = (b.h[k] - oo) / dd;
        if (t1 > t2) std::swap(t1, t2);
        lo = std::max(lo, t1);
        hi = std::min(hi, t2);
        if (lo > hi) return std::numeric_limits<double>::infinity();
    }
    return lo > 0 ? lo : std::numeric_limits<double>::infinity();
}

}  // namespace

struct tsyn_world {
    std::vector<Box> boxes;
    double lo[3], hi[3];   // extent of all geometry
    double pose[6];        // a default sensor pose inside the free space
    // 2-D bucket grid over x,y for box lookup
    double cell = 4.0;
    int gx = 1, gy = 1;
    std::vector<std::vector<int>> grid;
    double margin = 1.5;   // boxes are registered in every bucket their AABB +margin touches

    void finalize()
    {
        for (int a = 0; a < 3; ++a) { lo[a] = 1e300; hi[a] = -1e300; }
        for (auto& b : boxes)
            for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
        gx = std::max(1, (int)std::ceil((hi[0] - lo[0] + 2 * margin) / cell));
        gy = std::max(1, (int)std::ceil((hi[1] - lo[1] + 2 * margin) / cell));
        grid.assign((size_t)gx * gy, {});
        for (int i = 0; i < (int)boxes.size(); ++i) {
            const Box& b = boxes[i];
            int x0 = bucket(b.lo[0] - margin, 0), x1 = bucket(b.hi[0] + margin, 0);
            int y0 = bucket(b.lo[1] - margin, 1), y1 = bucket(b.hi[1] + margin, 1);
            for (int x = x0; x <= x1; ++x)
                for (int y = y0; y <= y1; ++y) grid[(size_t)y * gx + x].push_back(i);
        }
    }
    int bucket(double v, int axis) const
    {
        int n = axis == 0 ? gx : gy;
        int k = (int)std::floor((v - (lo[axis] - margin)) / cell);
        return std::min(std::max(k, 0), n - 1);
    }
    // Signed distance; exact within `margin` of any surface, clamped beyond.
    double sdf(const double p[3]) const
    {
        const auto& list = grid[(size_t)bucket(p[1], 1) * gx + bucket(p[0], 0)];
        double d = margin + 1.0;
        for (int i : list) d = std::min(d, box_sdf(boxes[i], p));
        return d;
    }
    double ray(const double o[3], const double dir[3], double max_range) const
    {
        double best = std::numeric_limits<double>::infinity();
        for (const auto& b : boxes) {
            // quick reject against the AABB
            double t = box_ray(b, o, dir);
            if (t < best) best = t;
        }
        return best <= max_range ? best : std::numeric_limits<double>::infinity();
    }
};

namespace {

void add_room_shell(tsyn_world& w, double x0, double y0, double z0, double sx, double sy, double sz, double t)
{
    // floor, ceiling, four walls (interior is [x0,x0+sx] x [y0,y0+sy] x [z0,z0+sz])
    w.boxes.push_back(make_box(x0 + sx / 2, y0 + sy / 2, z0 - t / 2, sx / 2 + t, sy / 2 + t, t / 2));
    w.boxes.push_back(make_box(x0 + sx / 2, y0 + sy / 2, z0 + sz + t / 2, sx / 2 + t, sy / 2 + t, t / 2));
    w.boxes.push_back(make_box(x0 - t / 2, y0 + sy / 2, z0 + sz / 2, t / 2, sy / 2 + t, sz / 2));
    w.boxes.push_back(make_box(x0 + sx + t / 2, y0 + sy / 2, z0 + sz / 2, t / 2, sy / 2 + t, sz / 2));
    w.boxes.push_back(make_box(x0 + sx / 2, y0 - t / 2, z0 + sz / 2, sx / 2, t / 2, sz / 2));
    w.boxes.push_back(make_box(x0 + sx / 2, y0 + sy + t / 2, z0 + sz / 2, sx / 2, t / 2, sz / 2));
}

// 20 x 20 x 4 m room: axis-aligned boxes plus 6 randomly oriented planes.
void build_room(tsyn_world& w, Rng& rng)
{
    const double x0 = 1.0, y0 = 1.0, z0 = 1.0, S = 20.0, H = 4.0;
    add_room_shell(w, x0, y0, z0, S, S, H, 0.2);
    for (int i = 0; i < 10; ++i) {
        double hx = rng.uniform(0.2, 0.9), hy = rng.uniform(0.2, 0.9), hz = rng.uniform(0.2, 0.8);
        double cx = rng.uniform(x0 + 2, x0 + S - 2), cy = rng.uniform(y0 + 2, y0 + S - 2);
        if (std::hypot(cx - 11.0, cy - 11.0) < 3.0) cx += 4.0;  // keep the sensor area clear
        w.boxes.push_back(make_box(cx, cy, z0 + hz, hx, hy, hz));
    }
    for (int i = 0; i < 6; ++i) {
        double cx = rng.uniform(x0 + 3, x0 + S - 3), cy = rng.uniform(y0 + 3, y0 + S - 3);
        if (std::hypot(cx - 11.0, cy - 11.0) < 3.5) cy += 5.0;
        double cz = rng.uniform(z0 + 1.0, z0 + H - 1.0);
        w.boxes.push_back(make_box(cx, cy, cz, rng.uniform(0.6, 1.6), 0.03, rng.uniform(0.5, 1.2),
                                   rng.uniform(-0.6, 0.6), rng.uniform(-0.6, 0.6), rng.uniform(-3.1, 3.1)));
    }
    w.pose[0] = 11.0; w.pose[1] = 11.0; w.pose[2] = z0 + 1.2;
    w.pose[3] = 0; w.pose[4] = 0; w.pose[5] = rng.uniform(-3.1, 3.1);
}

// 100 x 100 x 10 m building: two storeys of 10 m x 10 m rooms separated by
// walls with door openings, a central corridor, boxes and ramps.
void build_building(tsyn_world& w, Rng& rng)
{
    const double x0 = 1.0, y0 = 1.0, z0 = 1.0, S = 100.0, H = 10.0, t = 0.2, st = 5.0;
    add_room_shell(w, x0, y0, z0, S, S, H, 0.3);
    // intermediate floor slab with a stair well
    w.boxes.push_back(make_box(x0 + S / 2, y0 + S / 4 + 2, z0 + st, S / 2, S / 4 - 2, t / 2));
    w.boxes.push_back(make_box(x0 + S / 2, y0 + 3 * S / 4 - 2, z0 + st, S / 2, S / 4 - 2, t / 2));
    for (int storey = 0; storey < 2; ++storey) {
        double zb = z0 + storey * st, zh = st / 2;
        for (int k = 1; k < 10; ++k) {
            double xw = x0 + 10.0 * k;
            for (int seg = 0; seg < 10; ++seg) {  // walls along y with doors
                double ya = y0 + 10.0 * seg, yb = ya + 10.0;
                if (seg == 4 || seg == 5) continue;  // corridor
                double door = ya + rng.uniform(2.0, 7.0);
                w.boxes.push_back(make_box(xw, (ya + door - 0.5) / 2, zb + zh, t / 2, (door - 0.5 - ya) / 2, zh));
                w.boxes.push_back(make_box(xw, (door + 0.5 + yb) / 2, zb + zh, t / 2, (yb - door - 0.5) / 2, zh));
            }
        }
        for (int k = 1; k < 10; ++k) {
            if (k == 5) continue;
            double yw = y0 + 10.0 * k;
            for (int seg = 0; seg < 10; ++seg) {
                double xa = x0 + 10.0 * seg, xb = xa + 10.0;
                double door = xa + rng.uniform(2.0, 7.0);
                w.boxes.push_back(make_box((xa + door - 0.5) / 2, yw, zb + zh, (door - 0.5 - xa) / 2, t / 2, zh));
                w.boxes.push_back(make_box((door + 0.5 + xb) / 2, yw, zb + zh, (xb - door - 0.5) / 2, t / 2, zh));
            }
        }
        for (int i = 0; i < 120; ++i) {
            double hx = rng.uniform(0.2, 1.0), hy = rng.uniform(0.2, 1.0), hz = rng.uniform(0.2, 1.0);
            double cx = rng.uniform(x0 + 1.5, x0 + S - 1.5), cy = rng.uniform(y0 + 1.5, y0 + S - 1.5);
            if (std::fabs(cy - (y0 + S / 2)) < 3.0) continue;  // corridor stays clear
            w.boxes.push_back(make_box(cx, cy, zb + hz, hx, hy, hz, 0, 0, rng.uniform(-0.5, 0.5)));
        }
    }
    // ramps in the corridor
    for (int i = 0; i < 4; ++i) {
        double cx = x0 + 15 + 20 * i;
        w.boxes.push_back(make_box(cx, y0 + S / 2 + 2.5, z0 + 0.6, 3.0, 1.0, 0.1, 0.0, -0.2, 0.0));
    }
    w.pose[0] = x0 + S / 2 + 3.3; w.pose[1] = y0 + S / 2 - 0.4; w.pose[2] = z0 + 1.5;
    w.pose[3] = 0; w.pose[4] = 0; w.pose[5] = rng.uniform(-3.1, 3.1);
}

// 200 x 80 x 15 m warehouse with rows of shelving racks.
void build_warehouse(tsyn_world& w, Rng& rng)
{
    const double x0 = 1.0, y0 = 1.0, z0 = 1.0, SX = 200.0, SY = 80.0, H = 15.0;
    add_room_shell(w, x0, y0, z0, SX, SY, H, 0.3);
    for (int row = 0; row < 12; ++row) {
        double cy = y0 + 6 + row * 6.0;
        for (int seg = 0; seg < 8; ++seg) {
            double cx = x0 + 12 + seg * 24.0;
            double h = rng.uniform(4.0, 9.0);
            w.boxes.push_back(make_box(cx, cy, z0 + h / 2, 10.0, 0.6, h / 2));
            for (int lvl = 1; lvl < 4; ++lvl)
                w.boxes.push_back(make_box(cx, cy, z0 + lvl * h / 4, 10.2, 0.75, 0.04));
        }
    }
    for (int i = 0; i < 60; ++i)
        w.boxes.push_back(make_box(rng.uniform(x0 + 3, x0 + SX - 3), y0 + 3 + 6.0 * rng.uniform(0, 12) + 3.0,
                                   z0 + 0.6, 0.6, 0.6, 0.6, 0, 0, rng.uniform(-0.3, 0.3)));
    w.pose[0] = x0 + 40.5; w.pose[1] = y0 + 9.0; w.pose[2] = z0 + 1.5;
    w.pose[3] = 0; w.pose[4] = 0; w.pose[5] = 0.1;
}

// 500 x 8 x 6 m tunnel with ribs and pipes.
void build_tunnel(tsyn_world& w, Rng& rng)
{
    const double x0 = 1.0, y0 = 1.0, z0 = 1.0, L = 500.0, W = 8.0, H = 6.0;
    add_room_shell(w, x0, y0, z0, L, W, H, 0.3);
    for (double x = x0 + 5; x < x0 + L - 5; x += 10.0) {
        w.boxes.push_back(make_box(x, y0 + 0.15, z0 + H / 2, 0.25, 0.15, H / 2));
        w.boxes.push_back(make_box(x, y0 + W - 0.15, z0 + H / 2, 0.25, 0.15, H / 2));
        w.boxes.push_back(make_box(x, y0 + W / 2, z0 + H - 0.15, 0.25, W / 2, 0.15));
    }
    w.boxes.push_back(make_box(x0 + L / 2, y0 + 0.6, z0 + H - 1.0, L / 2, 0.2, 0.2));
    w.boxes.push_back(make_box(x0 + L / 2, y0 + W - 0.6, z0 + 0.8, L / 2, 0.25, 0.25));
    for (int i = 0; i < 80; ++i)
        w.boxes.push_back(make_box(rng.uniform(x0 + 2, x0 + L - 2), rng.uniform(y0 + 1.5, y0 + W - 1.5), z0 + 0.3,
                                   rng.uniform(0.2, 0.6), rng.uniform(0.2, 0.6), 0.3, 0, 0, rng.uniform(-1, 1)));
    w.pose[0] = x0 + 52.0; w.pose[1] = y0 + W / 2 + 0.3; w.pose[2] = z0 + 1.5;
    w.pose[3] = 0; w.pose[4] = 0; w.pose[5] = 0.05;
}

struct ChunkKey {
    int32_t x, y, z;
    bool operator==(const ChunkKey& o) const { return x == o.x && y == o.y && z == o.z; }
};

}  // namespace

extern "C" {

// kind: 0 room 20x20x4, 1 building 100x100x10, 2 warehouse 200x80x15, 3 tunnel 500x8x6
tsyn_world* tsyn_world_create(int kind, uint64_t seed)
{
    auto* w = new tsyn_world;
    Rng rng(seed);
    switch (kind) {
        case 0: build_room(*w, rng); break;
        case 1: build_building(*w, rng); break;
        case 2: build_warehouse(*w, rng); break;
        case 3: build_tunnel(*w, rng); break;
        default: delete w; return nullptr;
    }
    w->finalize();
    return w;
}

void tsyn_world_destroy(tsyn_world* w) { delete w; }

void tsyn_world_info(const tsyn_world* w, float lo[3], float hi[3], float pose[6], int32_t* n_boxes)
{
    for (int a = 0; a < 3; ++a) { lo[a] = (float)w->lo[a]; hi[a] = (float)w->hi[a]; }
    for (int a = 0; a < 6; ++a) pose[a] = (float)w->pose[a];
    *n_boxes = (int32_t)w->boxes.size();
}

float tsyn_world_sdf(const tsyn_world* w, float x, float y, float z)
{
    double p[3] = {x, y, z};
    return (float)w->sdf(p);
}

void tsyn_free(void* p) { std::free(p); }

// TSDF of the world at cell size voxel_mm, over the band |sdf| < band_m
// (weight 1 there, 0 elsewhere; value = round(sdf in mm) clamped to +-600).
// Cells live on the lattice x = i * voxel_mm (the reference's cell positions,
// map_util.h:111-120).  The band is returned as chunks of edge^3 cells: 3 ints
// of chunk coordinates and edge^3 raw uint32 cells each (index e*e*i + e*j + k,
// map_util.h:106).  Chunks are ordered by their "x_y_z" name as the map reader
// lists them.  Returns the chunk count; *pos_out / *raw_out are malloc'd.
size_t tsyn_tsdf_chunks(const tsyn_world* w, int voxel_mm, int edge, float band_m, int32_t** pos_out,
                        uint32_t** raw_out)
{
    const double r = voxel_mm * 0.001;
    const double reach = band_m + r * edge * 0.8660254 + 1e-6;  // brick half-diagonal
    int64_t lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = (int64_t)std::floor((w->lo[a] - band_m) / r / edge) - 0;
        hi[a] = (int64_t)std::floor((w->hi[a] + band_m) / r / edge);
    }
    // candidate chunks: test the centre sdf
    std::vector<ChunkKey> keys;
    int64_t nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    std::vector<uint8_t> keep((size_t)(nx * ny * nz), 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t id = 0; id < nx * ny * nz; ++id) {
        int64_t cx = lo[0] + id % nx, cy = lo[1] + (id / nx) % ny, cz = lo[2] + id / (nx * ny);
        double c[3] = {(cx * edge + (edge - 1) * 0.5) * r, (cy * edge + (edge - 1) * 0.5) * r,
                       (cz * edge + (edge - 1) * 0.5) * r};
        if (std::fabs(w->sdf(c)) < reach) keep[id] = 1;
    }
    for (int64_t id = 0; id < nx * ny * nz; ++id)
        if (keep[id]) keys.push_back({(int32_t)(lo[0] + id % nx), (int32_t)(lo[1] + (id / nx) % ny), (int32_t)(lo[2] + id / (nx * ny))});
    const size_t cells = (size_t)edge * edge * edge;
    std::vector<uint8_t> nonempty(keys.size(), 0);
    uint32_t* raw = (uint32_t*)std::calloc(keys.size() * cells + 1, sizeof(uint32_t));
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t k = 0; k < (int64_t)keys.size(); ++k) {
        uint32_t* out = raw + (size_t)k * cells;
        bool any = false;
        for (int i = 0; i < edge; ++i)
            for (int j = 0; j < edge; ++j)
                for (int l = 0; l < edge; ++l) {
                    double p[3] = {(double)(keys[k].x * edge + i) * r, (double)(keys[k].y * edge + j) * r,
                                   (double)(keys[k].z * edge + l) * r};
                    double d = w->sdf(p);
                    if (std::fabs(d) >= band_m) continue;
                    long mm = std::lround(d * 1000.0);
                    mm = std::max(-600l, std::min(600l, mm));
                    uint16_t v = (uint16_t)(int16_t)mm, wt = 1;
                    out[(size_t)edge * edge * i + (size_t)edge * j + l] = (uint32_t)v | ((uint32_t)wt << 16);
                    any = true;
                }
        nonempty[k] = any;
    }
    // compact and order by name
    std::vector<size_t> order;
    for (size_t k = 0; k < keys.size(); ++k)
        if (nonempty[k]) order.push_back(k);
    std::vector<std::string> names(keys.size());
    for (size_t k : order) {
        char buf[48];
        std::snprintf(buf, sizeof(buf), "%d_%d_%d", keys[k].x, keys[k].y, keys[k].z);
        names[k] = buf;
    }
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return names[a] < names[b]; });
    int32_t* pos = (int32_t*)std::malloc(sizeof(int32_t) * 3 * (order.size() + 1));
    uint32_t* packed = (uint32_t*)std::malloc(sizeof(uint32_t) * (order.size() * cells + 1));
    for (size_t t = 0; t < order.size(); ++t) {
        size_t k = order[t];
        pos[3 * t] = keys[k].x; pos[3 * t + 1] = keys[k].y; pos[3 * t + 2] = keys[k].z;
        std::memcpy(packed + t * cells, raw + k * cells, sizeof(uint32_t) * cells);
    }
    std::free(raw);
    *pos_out = pos;
    *raw_out = packed;
    return order.size();
}

// Ray-cast a rings x cols spinning LiDAR from pose6 = (x,y,z,roll,pitch,yaw) of
// the sensor.  Elevations are uniform in [vmin_deg, vmax_deg].  Ranges get
// Gaussian noise (sigma) and each return is dropped with probability dropout;
// rays with no hit within max_range or closer than min_range are skipped.
// Points are written in the sensor frame in ring-major order with their ring.
size_t tsyn_scan(const tsyn_world* w, const float pose6[6], int rings, int cols, float vmin_deg, float vmax_deg,
                 float min_range, float max_range, float sigma, float dropout, uint64_t seed, float* xyz_out,
                 int16_t* ring_out)
{
    double R[3][3];
    rot_rpy(pose6[3], pose6[4], pose6[5], R);  // R rows: world->local; columns: local axes in world
    const double o[3] = {pose6[0], pose6[1], pose6[2]};
    std::vector<double> range((size_t)rings * cols);
#pragma omp parallel for schedule(dynamic, 1)
    for (int ring = 0; ring < rings; ++ring) {
        double el = (rings == 1 ? 0.5 * (vmin_deg + vmax_deg)
                                : vmin_deg + (vmax_deg - vmin_deg) * ring / (rings - 1)) * M_PI / 180.0;
        for (int c = 0; c < cols; ++c) {
            double az = 2 * M_PI * c / cols;
            double dl[3] = {std::cos(el) * std::cos(az), std::cos(el) * std::sin(az), std::sin(el)};
            double dw[3];
            for (int a = 0; a < 3; ++a) dw[a] = R[0][a] * dl[0] + R[1][a] * dl[1] + R[2][a] * dl[2];
            range[(size_t)ring * cols + c] = w->ray(o, dw, max_range);
        }
    }
    Rng rng(seed);
    size_t n = 0;
    for (int ring = 0; ring < rings; ++ring) {
        double el = (rings == 1 ? 0.5 * (vmin_deg + vmax_deg)
                                : vmin_deg + (vmax_deg - vmin_deg) * ring / (rings - 1)) * M_PI / 180.0;
        for (int c = 0; c < cols; ++c) {
            double t = range[(size_t)ring * cols + c];
            double noise = rng.normal() * sigma;
            double drop = rng.uniform();
            if (!std::isfinite(t)) continue;
            if (drop < dropout) continue;
            t += noise;
            if (t < min_range || t > max_range) continue;
            double az = 2 * M_PI * c / cols;
            xyz_out[3 * n] = (float)(t * std::cos(el) * std::cos(az));
            xyz_out[3 * n + 1] = (float)(t * std::cos(el) * std::sin(az));
            xyz_out[3 * n + 2] = (float)(t * std::sin(el));
            ring_out[n] = (int16_t)ring;
            ++n;
        }
    }
    return n;
}

// Scan reduction of the reference's scan preparation (tsdf_evaluator.cpp:304-376):
// points closer than 1 m are dropped, one point is kept per (ring, cell of
// edge `cell`) -- the first in scan order --, and the kept points are ordered by
// ring, then by scan index.  The kept point is the original, not the cell
// centre.  Returns the number of points written to out.
size_t tsyn_reduce_scan(const float* xyz, const int16_t* ring, size_t n, float cell, float* out)
{
    struct Key {
        int16_t ring;
        float cx, cy, cz;
        bool operator==(const Key& o) const { return ring == o.ring && cx == o.cx && cy == o.cy && cz == o.cz; }
    };
    struct H {
        size_t operator()(const Key& k) const
        {
            long long v = ((long long)(k.cx * 1000) << 32) ^ ((long long)(k.cy * 1000) << 16) ^ (long long)(k.cz * 1000);
            return std::hash<long long>()(v) ^ (size_t)k.ring;
        }
    };
    std::unordered_set<Key, H> seen;
    std::vector<std::pair<std::pair<int, size_t>, size_t>> kept;
    float half = cell / 2;
    for (size_t i = 0; i < n; ++i) {
        float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        float dist = std::sqrt(x * x + y * y + z * z);
        if (dist < 1.0f) continue;
        Key k{ring[i], (float)(std::floor(x / cell) * cell + half), (float)(std::floor(y / cell) * cell + half),
              (float)(std::floor(z / cell) * cell + half)};
        if (seen.insert(k).second) kept.push_back({{(int)ring[i], i}, i});
    }
    std::sort(kept.begin(), kept.end());
    for (size_t t = 0; t < kept.size(); ++t) std::memcpy(out + 3 * t, xyz + 3 * kept[t].second, sizeof(float) * 3);
    return kept.size();
}

// Keeps exactly m of the n points (n >= m) with a seeded choice, in their order.
void tsyn_subsample_ordered(const float* xyz, size_t n, size_t m, uint64_t seed, float* out)
{
    std::vector<size_t> idx(n);
    for (size_t i = 0; i < n; ++i) idx[i] = i;
    Rng rng(seed);
    for (size_t i = 0; i < m && i < n; ++i) {
        size_t j = i + (size_t)(rng.uniform() * (double)(n - i));
        if (j >= n) j = n - 1;
        std::swap(idx[i], idx[j]);
    }
    std::sort(idx.begin(), idx.begin() + std::min(m, n));
    for (size_t t = 0; t < m && t < n; ++t) std::memcpy(out + 3 * t, xyz + 3 * idx[t], sizeof(float) * 3);
}

// P particles (AoS x,y,z,roll,pitch,yaw,weight) Gaussian around center6 with
// sigma_xyz (m) and sigma_rpy (rad); weights 1/P.
void tsyn_particles_gaussian(const float center6[6], float sigma_xyz, float sigma_rpy, size_t P, uint64_t seed,
                             float* out7)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)P; ++i) {
        Rng rng(seed ^ (0x51ED2701ull * (uint64_t)(i + 1)));
        for (int a = 0; a < 3; ++a) out7[7 * i + a] = (float)(center6[a] + sigma_xyz * rng.normal());
        for (int a = 3; a < 6; ++a) out7[7 * i + a] = (float)(center6[a] + sigma_rpy * rng.normal());
        out7[7 * i + 6] = (float)(1.0 / (double)P);
    }
}

// P particles uniform over free space: positions with sdf >= clearance inside
// the world extent (z within [zlo, zhi]), yaw uniform, roll/pitch uniform in
// +-rp_max.
void tsyn_particles_free_space(const tsyn_world* w, float clearance, float zlo, float zhi, float rp_max, size_t P,
                               uint64_t seed, float* out7)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)P; ++i) {
        Rng rng(seed ^ (0x2545F491ull * (uint64_t)(i + 1)));
        for (int tries = 0; tries < 10000; ++tries) {
            double p[3] = {rng.uniform(w->lo[0], w->hi[0]), rng.uniform(w->lo[1], w->hi[1]), rng.uniform(zlo, zhi)};
            if (w->sdf(p) >= clearance || tries == 9999) {
                for (int a = 0; a < 3; ++a) out7[7 * i + a] = (float)p[a];
                break;
            }
        }
        out7[7 * i + 3] = (float)rng.uniform(-rp_max, rp_max);
        out7[7 * i + 4] = (float)rng.uniform(-rp_max, rp_max);
        out7[7 * i + 5] = (float)rng.uniform(-M_PI, M_PI);
        out7[7 * i + 6] = (float)(1.0 / (double)P);
    }
}

}  // extern "C"
