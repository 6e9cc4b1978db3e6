// lp_synth.cpp — seeded synthetic spinning-LiDAR scans (host code, liblp_synth.so).
//
// Stands in for the reference's KITTI-style HDL-64E frames (data/*.pcd). Rays are cast from a
// sensor at the origin against a ground surface 1.73 m below it and against boxes, vertical
// cylinders and a wall; returns are emitted ring by ring, top (highest elevation) ring first,
// each ring swept in ascending azimuth from 0 to 2*pi, which is the organised order the
// reference's ring partition (dataloader.cpp:68-137) recovers rings from.
//
// Workloads (seed = 1000 * workload + scan index):
//   1  64 rings +2.0..-24.8 deg, 2048 bins, 80 m, flat ground (height noise 0.02 m), 20 yawed
//      4.5x1.8x1.5 m boxes in the 5-40 m annulus, 8 cylinders r 0.15 m h 4 m, a 30 x 3 m wall at
//      25 m, range noise 0.02 m, 10 % dropout, intensity U[0,1]            (~110k points)
//   2  128 rings +15..-25 deg, undulating ground + 4 deg slope beyond 20 m, 80 boxes with sides
//      U[0.5,6] m, 40 cylinders, 2 % of returns moved 0.1-0.5 m below the ground (~230k points)
//   3  per scan: rings {32,64,128}, bins {1024,2048,4096}, return rate U[0.3,1], obstacles
//      U[10,200], ground flat / sloped / undulating (32 rings use +2..-24.8 deg)
//   4  workload-2 geometry at 16384 bins, 950,000 returns drawn without replacement, plus
//      50,000 clutter points within 15 m (density ~ 1/r), shuffled: 1,000,000 points
//   5  serving mix: like 3 (scan sizes ~30k-500k)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace
{
struct Rng
{
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double uni() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uni(double a, double b) { return a + (b - a) * uni(); }
    double normal()
    {
        double u1 = uni();
        if (u1 < 1e-300)
            u1 = 1e-300;
        const double u2 = uni();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }
};

struct Box
{
    double cx, cy, cz0, yaw, hl, hw, h; // centre, bottom z, yaw, half length/width, height
    double c, s;
};
struct Cyl
{
    double cx, cy, cz0, r, h;
};

enum Ground
{
    FLAT = 0,
    SLOPED = 1,
    UNDULATING = 2
};

struct Scene
{
    int ground;
    double sensor_h;
    double slope_start, slope_tan;
    std::vector<Box> boxes;
    std::vector<Cyl> cyls;

    double groundZ(double x, double y) const
    {
        double z = -sensor_h;
        if (ground == UNDULATING)
            z += 0.3 * std::sin(2.0 * M_PI * x / 30.0) + 0.02 * std::sin(2.0 * M_PI * y / 7.0);
        if (ground != FLAT)
        {
            const double rho = std::sqrt(x * x + y * y);
            if (rho > slope_start)
                z += slope_tan * (rho - slope_start);
        }
        return z;
    }
};

bool hitBox(const Box& b, const double d[3], double& t)
{
    // ray origin (0,0,0) in the box frame
    const double ox = -b.cx, oy = -b.cy;
    const double lx = b.c * ox + b.s * oy, ly = -b.s * ox + b.c * oy;
    const double dx = b.c * d[0] + b.s * d[1], dy = -b.s * d[0] + b.c * d[1];
    double t0 = 0.0, t1 = 1e30;
    const double o[3] = {lx, ly, 0.0};
    const double dd[3] = {dx, dy, d[2]};
    const double lo[3] = {-b.hl, -b.hw, b.cz0};
    const double hi[3] = {b.hl, b.hw, b.cz0 + b.h};
    for (int k = 0; k < 3; ++k)
    {
        if (std::fabs(dd[k]) < 1e-12)
        {
            if (o[k] < lo[k] || o[k] > hi[k])
                return false;
            continue;
        }
        double a = (lo[k] - o[k]) / dd[k], c = (hi[k] - o[k]) / dd[k];
        if (a > c)
            std::swap(a, c);
        t0 = std::max(t0, a);
        t1 = std::min(t1, c);
        if (t0 > t1)
            return false;
    }
    t = t0;
    return t0 > 0.0;
}

bool hitCyl(const Cyl& cy, const double d[3], double& t)
{
    const double a = d[0] * d[0] + d[1] * d[1];
    if (a < 1e-12)
        return false;
    const double b = -2.0 * (d[0] * cy.cx + d[1] * cy.cy);
    const double c = cy.cx * cy.cx + cy.cy * cy.cy - cy.r * cy.r;
    const double disc = b * b - 4 * a * c;
    if (disc < 0)
        return false;
    const double tt = (-b - std::sqrt(disc)) / (2 * a);
    if (tt <= 0)
        return false;
    const double z = tt * d[2];
    if (z < cy.cz0 || z > cy.cz0 + cy.h)
        return false;
    t = tt;
    return true;
}

// Returns the ground hit distance along the ray (or < 0 for none) within [0, tmax].
double hitGround(const Scene& sc, const double d[3], double tmax)
{
    if (sc.ground == FLAT)
    {
        if (d[2] >= -1e-9)
            return -1.0;
        const double t = -sc.sensor_h / d[2];
        return t <= tmax ? t : -1.0;
    }
    auto f = [&](double t) { return t * d[2] - sc.groundZ(t * d[0], t * d[1]); };
    double prev_t = 0.0, prev_f = f(0.0);
    double t = 0.5;
    while (t <= tmax)
    {
        const double ft = f(t);
        if ((ft < 0) != (prev_f < 0))
        {
            double a = prev_t, b = t;
            for (int it = 0; it < 40; ++it)
            {
                const double m = 0.5 * (a + b);
                if ((f(m) < 0) == (prev_f < 0))
                    a = m;
                else
                    b = m;
            }
            return 0.5 * (a + b);
        }
        prev_t = t;
        prev_f = ft;
        t += std::max(0.1, 0.01 * t);
    }
    return -1.0;
}

struct Params
{
    int rings, bins;
    double el_up, el_down, max_range;
    int ground;
    double ground_sigma, range_sigma, return_rate;
    int n_boxes;
    int fixed_box; // 1: 4.5x1.8x1.5 boxes; 0: sides U[0.5, 6]
    int n_cyl;
    int wall;
    double artifact_frac;
    int target_returns; // >0: keep exactly this many returns (drawn without replacement)
    int clutter;        // clutter points added after the returns
    int shuffle;
};

Params preset(int workload, int scan, Rng& rng)
{
    Params p{64, 2048, 2.0, -24.8, 80.0, FLAT, 0.02, 0.02, 0.9, 20, 1, 8, 1, 0.0, 0, 0, 0};
    if (workload == 2 || workload == 4)
    {
        p.rings = 128;
        p.el_up = 15.0;
        p.el_down = -25.0;
        p.ground = UNDULATING;
        p.n_boxes = 80;
        p.fixed_box = 0;
        p.n_cyl = 40;
        p.artifact_frac = 0.02;
        if (workload == 4)
        {
            p.bins = 16384;
            p.target_returns = 950000;
            p.clutter = 50000;
            p.shuffle = 1;
        }
    }
    else if (workload == 3 || workload == 5)
    {
        static const int R[3] = {32, 64, 128};
        static const int Wb[3] = {1024, 2048, 4096};
        p.rings = R[rng.next() % 3];
        p.bins = Wb[rng.next() % 3];
        if (p.rings == 128)
        {
            p.el_up = 15.0;
            p.el_down = -25.0;
        }
        p.return_rate = rng.uni(0.3, 1.0);
        const int obstacles = 10 + static_cast<int>(rng.next() % 191);
        p.n_boxes = (obstacles * 2) / 3;
        p.n_cyl = obstacles - p.n_boxes;
        p.fixed_box = 0;
        p.ground = static_cast<int>(rng.next() % 3);
        p.wall = static_cast<int>(rng.next() % 2);
    }
    (void)scan;
    return p;
}

void buildScene(const Params& p, Rng& rng, Scene& sc)
{
    sc.ground = p.ground;
    sc.sensor_h = 1.73;
    sc.slope_start = 20.0;
    sc.slope_tan = std::tan(4.0 * M_PI / 180.0);
    auto place = [&](double& x, double& y) {
        const double r = std::sqrt(rng.uni(25.0, 1600.0)); // area-uniform in the 5-40 m annulus
        const double a = rng.uni(0.0, 2.0 * M_PI);
        x = r * std::cos(a);
        y = r * std::sin(a);
    };
    for (int i = 0; i < p.n_boxes; ++i)
    {
        Box b;
        place(b.cx, b.cy);
        b.yaw = rng.uni(0.0, 2.0 * M_PI);
        if (p.fixed_box)
        {
            b.hl = 2.25;
            b.hw = 0.9;
            b.h = 1.5;
        }
        else
        {
            b.hl = 0.5 * rng.uni(0.5, 6.0);
            b.hw = 0.5 * rng.uni(0.5, 6.0);
            b.h = rng.uni(0.5, 6.0);
        }
        b.cz0 = sc.groundZ(b.cx, b.cy);
        b.c = std::cos(b.yaw);
        b.s = std::sin(b.yaw);
        sc.boxes.push_back(b);
    }
    for (int i = 0; i < p.n_cyl; ++i)
    {
        Cyl c;
        place(c.cx, c.cy);
        c.r = 0.15;
        c.h = 4.0;
        c.cz0 = sc.groundZ(c.cx, c.cy);
        sc.cyls.push_back(c);
    }
    if (p.wall)
    {
        Box w;
        const double a = rng.uni(0.0, 2.0 * M_PI);
        w.cx = 25.0 * std::cos(a);
        w.cy = 25.0 * std::sin(a);
        w.yaw = a + 0.5 * M_PI; // length perpendicular to the radial direction
        w.hl = 15.0;
        w.hw = 0.1;
        w.h = 3.0;
        w.cz0 = sc.groundZ(w.cx, w.cy);
        w.c = std::cos(w.yaw);
        w.s = std::sin(w.yaw);
        sc.boxes.push_back(w);
    }
}

struct Ret
{
    float x, y, z, i;
    uint16_t ring;
};

// Casts one ring; appends returns in azimuth order. Per-ray randomness comes from a generator
// seeded by (scan seed, ring) so that rings can be cast in parallel deterministically.
void castRing(const Params& p, const Scene& sc, uint64_t seed, int k, std::vector<Ret>& out)
{
    Rng rng(seed * 1315423911ULL + static_cast<uint64_t>(k) + 7);
    const double el = (p.el_up + (p.el_down - p.el_up) * (p.rings > 1 ? static_cast<double>(k) / (p.rings - 1) : 0.0)) *
                      M_PI / 180.0;
    const uint16_t ring = static_cast<uint16_t>(p.rings - 1 - k);
    for (int j = 0; j < p.bins; ++j)
    {
        const double az = (j + 0.5) * 2.0 * M_PI / p.bins;
        const double d[3] = {std::cos(el) * std::cos(az), std::cos(el) * std::sin(az), std::sin(el)};
        double tbest = p.max_range;
        bool any = false, is_ground = false;
        double t;
        for (const auto& b : sc.boxes)
            if (hitBox(b, d, t) && t < tbest)
            {
                tbest = t;
                any = true;
            }
        for (const auto& c : sc.cyls)
            if (hitCyl(c, d, t) && t < tbest)
            {
                tbest = t;
                any = true;
            }
        const double tg = hitGround(sc, d, tbest);
        if (tg > 0 && tg < tbest)
        {
            tbest = tg;
            any = true;
            is_ground = true;
        }
        const double u_drop = rng.uni();
        const double n_range = rng.normal();
        const double n_height = rng.normal();
        const double u_art = rng.uni();
        const double u_depth = rng.uni();
        const double inten = rng.uni();
        if (!any || u_drop >= p.return_rate)
            continue;
        const double tr = tbest + p.range_sigma * n_range;
        double x = tr * d[0], y = tr * d[1], z = tr * d[2];
        if (is_ground)
            z += p.ground_sigma * n_height;
        if (u_art < p.artifact_frac)
            z = sc.groundZ(x, y) - (0.1 + 0.4 * u_depth);
        out.push_back({static_cast<float>(x), static_cast<float>(y), static_cast<float>(z),
                       static_cast<float>(inten), ring});
    }
}

void generate(int workload, int scan, std::vector<Ret>& out, Params& p)
{
    const uint64_t seed = 1000ULL * static_cast<uint64_t>(workload) + static_cast<uint64_t>(scan);
    Rng rng(seed);
    p = preset(workload, scan, rng);
    Scene sc;
    buildScene(p, rng, sc);
    std::vector<std::vector<Ret>> per(p.rings);
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned w = 0; w < hw; ++w)
        th.emplace_back([&, w] {
            for (int k = static_cast<int>(w); k < p.rings; k += static_cast<int>(hw))
                castRing(p, sc, seed, k, per[k]);
        });
    for (auto& t : th)
        t.join();
    out.clear();
    for (const auto& r : per)
        out.insert(out.end(), r.begin(), r.end());
    if (p.target_returns > 0 && static_cast<int>(out.size()) > p.target_returns)
    {
        // keep a uniformly drawn subset of exactly target_returns, in their original order
        std::vector<uint8_t> keep(out.size(), 0);
        size_t need = static_cast<size_t>(p.target_returns);
        for (size_t i = 0; i < out.size() && need; ++i)
        {
            const size_t left = out.size() - i;
            if (rng.uni() * static_cast<double>(left) < static_cast<double>(need))
            {
                keep[i] = 1;
                --need;
            }
        }
        size_t w = 0;
        for (size_t i = 0; i < out.size(); ++i)
            if (keep[i])
                out[w++] = out[i];
        out.resize(w);
    }
    for (int c = 0; c < p.clutter; ++c)
    {
        const double r = 15.0 * std::sqrt(rng.uni());
        const double zc = rng.uni(-1.0, 1.0);
        const double a = rng.uni(0.0, 2.0 * M_PI);
        const double s = std::sqrt(1.0 - zc * zc);
        out.push_back({static_cast<float>(r * s * std::cos(a)), static_cast<float>(r * s * std::sin(a)),
                       static_cast<float>(r * zc), static_cast<float>(rng.uni()), 0});
    }
    if (p.shuffle)
    {
        for (size_t i = out.size(); i > 1; --i)
        {
            const size_t j = static_cast<size_t>(rng.next() % i);
            std::swap(out[i - 1], out[j]);
        }
    }
}
} // namespace

extern "C" {

// Scan shape for (workload, scan): rings, bins, elevation up/down (deg). Cheap (no casting).
void lp_synth_shape(int32_t workload, int32_t scan, int32_t* rings, int32_t* bins, float* el_up, float* el_down)
{
    const uint64_t seed = 1000ULL * static_cast<uint64_t>(workload) + static_cast<uint64_t>(scan);
    Rng rng(seed);
    const Params p = preset(workload, scan, rng);
    *rings = p.rings;
    *bins = p.bins;
    *el_up = static_cast<float>(p.el_up);
    *el_down = static_cast<float>(p.el_down);
}

// Upper bound on the number of points lp_synth_scan can return for (workload, scan).
uint32_t lp_synth_capacity(int32_t workload, int32_t scan)
{
    const uint64_t seed = 1000ULL * static_cast<uint64_t>(workload) + static_cast<uint64_t>(scan);
    Rng rng(seed);
    const Params p = preset(workload, scan, rng);
    return static_cast<uint32_t>(p.rings) * static_cast<uint32_t>(p.bins) + static_cast<uint32_t>(p.clutter);
}

// Generates scan `scan` of workload `workload`: xyzi (capacity x 4 floats) and the true ring of
// each return (0 for clutter). Returns the point count, or 0 if capacity is too small.
uint32_t lp_synth_scan(int32_t workload, int32_t scan, float* xyzi, uint16_t* ring, uint32_t capacity)
{
    std::vector<Ret> pts;
    Params p;
    generate(workload, scan, pts, p);
    if (pts.size() > capacity)
        return 0;
    for (size_t i = 0; i < pts.size(); ++i)
    {
        xyzi[4 * i] = pts[i].x;
        xyzi[4 * i + 1] = pts[i].y;
        xyzi[4 * i + 2] = pts[i].z;
        xyzi[4 * i + 3] = pts[i].i;
        if (ring)
            ring[i] = pts[i].ring;
    }
    return static_cast<uint32_t>(pts.size());
}
}
