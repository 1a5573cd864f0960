// Host-side solver entry points around the 2-opt path: TSPLIB parse, start
// tours and the tour check.  No GPU is needed for any function in this file.
//
//   logo_read_tsplib   ≙ readFileCoords       src/utils/tsp_loader.c:49-162
//   logo_nn_tour       ≙ initRoute_KD_NN      src/utils/kdtree_utils.c:279-301
//   logo_mf_tour       ≙ multipleFragment_KD  src/utils/kdtree_utils.c:56-242
//   logo_random_tour   ≙ routeInit(SHUFFLE)   src/utils/construction.c:129-137
//   logo_check_tour    ≙ checkTour            src/utils/construction.c:152-183
//   logo_read_tour     ≙ routeInitFromFile    src/utils/common.c:109-128
//   logo_write_tour    ≙ saveRouteToAFile     src/utils/common.c:144-192
//   logo_tsplib_info   (no counterpart: the reference reads every file as EUC_2D)
//
// Compiled with -ffp-contract=off: the nearest-neighbour search compares
// double distances and must not change with the host's FMA contraction.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include "../../include/logo_gpu.h"

namespace {

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform bucket grid over the bounding box with live-item lists per cell;
// nearest-neighbour queries scan square rings of cells outward and stop once
// a ring's closest possible point is farther than the best found.
class NNGrid {
public:
    NNGrid(const logo_xy* p, uint32_t n) : p_(p), n_(n) {
        double x0 = p[0].x, x1 = p[0].x, y0 = p[0].y, y1 = p[0].y;
        for (uint32_t k = 1; k < n; ++k) {
            x0 = std::min(x0, (double)p[k].x); x1 = std::max(x1, (double)p[k].x);
            y0 = std::min(y0, (double)p[k].y); y1 = std::max(y1, (double)p[k].y);
        }
        x0_ = x0;
        y0_ = y0;
        const double w = std::max(x1 - x0, 1e-30), h = std::max(y1 - y0, 1e-30);
        const double target = std::max(1.0, n / 2.0);
        double cell = std::sqrt(w * h / target);
        if (!(cell > 0)) cell = std::max(w, h);
        gw_ = (uint32_t)std::min<double>(4096.0, std::floor(w / cell) + 1);
        gh_ = (uint32_t)std::min<double>(4096.0, std::floor(h / cell) + 1);
        cw_ = w / gw_;
        ch_ = h / gh_;
        start_.assign((size_t)gw_ * gh_ + 1, 0);
        count_.assign((size_t)gw_ * gh_, 0);
        items_.resize(n);
        pos_.resize(n);
        cell_.resize(n);
        for (uint32_t k = 0; k < n; ++k) {
            cell_[k] = cell_of(p[k].x, p[k].y);
            count_[cell_[k]]++;
        }
        for (size_t c = 0; c < count_.size(); ++c) start_[c + 1] = start_[c] + count_[c];
        std::fill(count_.begin(), count_.end(), 0);
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t c = cell_[k];
            pos_[k] = start_[c] + count_[c]++;
            items_[pos_[k]] = k;
        }
        live_cells_ = 0;
        for (uint32_t c : count_) live_cells_ += c ? 1 : 0;
    }

    // Nearest live city to (px, py) by double Euclidean distance; ties go to
    // the lower id.  Cities skip_a and skip_b are passed over.
    uint32_t nearest(double px, double py, uint32_t skip_a = UINT32_MAX,
                     uint32_t skip_b = UINT32_MAX) const {
        uint32_t cx, cy;
        cell_xy(px, py, cx, cy);
        double best = INFINITY;
        uint32_t besti = UINT32_MAX;
        const uint32_t maxr = std::max(gw_, gh_);
        const double step = std::min(cw_, ch_);
        for (uint32_t r = 0; r <= maxr; ++r) {
            if (besti != UINT32_MAX && ((double)r - 1.0) * step > best) break;
            const int64_t xa = (int64_t)cx - r, xb = (int64_t)cx + r;
            const int64_t ya = (int64_t)cy - r, yb = (int64_t)cy + r;
            for (int64_t y = std::max<int64_t>(ya, 0); y <= std::min<int64_t>(yb, gh_ - 1); ++y) {
                if (y == ya || y == yb) {  // full row of the ring
                    for (int64_t x = std::max<int64_t>(xa, 0);
                         x <= std::min<int64_t>(xb, gw_ - 1); ++x)
                        scan_cell((size_t)y * gw_ + (size_t)x, px, py, skip_a, skip_b, best,
                                  besti);
                } else {  // only the two side cells
                    if (xa >= 0)
                        scan_cell((size_t)y * gw_ + (size_t)xa, px, py, skip_a, skip_b, best,
                                  besti);
                    if (xb != xa && xb < (int64_t)gw_)
                        scan_cell((size_t)y * gw_ + (size_t)xb, px, py, skip_a, skip_b, best,
                                  besti);
                }
            }
        }
        return besti;
    }

    void remove(uint32_t id) {
        const uint32_t c = cell_[id];
        const uint32_t last = start_[c] + count_[c] - 1;
        const uint32_t moved = items_[last];
        items_[pos_[id]] = moved;
        pos_[moved] = pos_[id];
        items_[last] = id;
        pos_[id] = last;
        count_[c]--;
    }

private:
    void scan_cell(size_t c, double px, double py, uint32_t skip_a, uint32_t skip_b,
                   double& best, uint32_t& besti) const {
        for (uint32_t t = 0; t < count_[c]; ++t) {
            const uint32_t id = items_[start_[c] + t];
            if (id == skip_a || id == skip_b) continue;
            const double dx = px - (double)p_[id].x, dy = py - (double)p_[id].y;
            const double d = std::sqrt(dx * dx + dy * dy);
            if (d < best || (d == best && id < besti)) {
                best = d;
                besti = id;
            }
        }
    }
    uint32_t cell_of(double x, double y) const {
        uint32_t cx, cy;
        cell_xy(x, y, cx, cy);
        return cy * gw_ + cx;
    }
    void cell_xy(double x, double y, uint32_t& cx, uint32_t& cy) const {
        double fx = (x - x0_) / cw_, fy = (y - y0_) / ch_;
        cx = fx <= 0 ? 0 : (uint32_t)std::min<double>(gw_ - 1, std::floor(fx));
        cy = fy <= 0 ? 0 : (uint32_t)std::min<double>(gh_ - 1, std::floor(fy));
    }
    const logo_xy* p_;
    uint32_t n_;
    double x0_, y0_, cw_, ch_;
    uint32_t gw_, gh_;
    std::vector<uint32_t> start_, count_, items_, pos_, cell_;
    uint32_t live_cells_;
};

// Host threads for the independent per-city queries of the start tour and
// neighbour-list builders: none below 20,000 cities, else the machine's
// (at most 16), or LOGO_HOST_THREADS when set.  Results do not depend on it.
unsigned host_threads(uint32_t n) {
    if (n < 20000) return 1;
    if (const char* e = std::getenv("LOGO_HOST_THREADS")) {
        const long v = std::strtol(e, nullptr, 10);
        return v < 1 ? 1u : (v > 64 ? 64u : (unsigned)v);
    }
    const unsigned hw = std::thread::hardware_concurrency();
    return hw < 1 ? 1u : (hw > 16 ? 16u : hw);
}

// nint(|a - b|) as an int: the per-edge distance in binary32 (this file is
// compiled without FMA contraction), truncated like the reference's
// fragment.distance (src/defs.h:201-205, from calculateDistance2D,
// src/headers.h:127-133).
int nint_dist(const logo_xy& a, const logo_xy& b) {
    const float dx = a.x - b.x, dy = a.y - b.y;
    return (int)(std::sqrt(dx * dx + dy * dy) + 0.5f);
}

// Greedy-edge ("multiple fragment") start tour, following the steps of
// multipleFragment_KD (src/utils/kdtree_utils.c:56-242) so that equal
// distances leave the priority queue in the same order: a max-heap (by
// std::priority_queue) of (nint distance to the current nearest valid
// neighbour, city); the top city x joins its neighbour y when y still has
// degree < 2 and is not the far end of x's own fragment, otherwise x's
// neighbour is looked up again among the cities of degree < 2 other than x
// and that far end, and x is pushed back.  Cities of degree 2 leave the
// search grid.  After n - 1 joins the path is listed from city 0: first the
// side of the neighbour city 0 was joined to first (reversed), then 0, then
// the side of its second neighbour.
struct Fragment {
    int distance;
    uint32_t id;
};
struct LaterFragment {  // the heap's top is the shortest distance
    bool operator()(const Fragment& a, const Fragment& b) const {
        return a.distance > b.distance;
    }
};

void mf_tour(const logo_xy* p, uint32_t n, uint32_t* route) {
    if (n <= 2) {
        for (uint32_t k = 0; k < n; ++k) route[k] = k;
        return;
    }
    NNGrid grid(p, n);
    std::vector<uint8_t> degree(n, 0);
    std::vector<uint32_t> link(n), tail(n);
    std::vector<int64_t> first(n, -1), second(n, -1);  // neighbours in join order
    std::priority_queue<Fragment, std::vector<Fragment>, LaterFragment> pq;
    // every city's first link is a query on the full grid, independent of
    // the others: split over host threads (the queue is then filled in
    // city order, as before)
    {
        auto links = [&](uint32_t lo, uint32_t hi) {
            for (uint32_t i = lo; i < hi; ++i) link[i] = grid.nearest(p[i].x, p[i].y, i);
        };
        const unsigned nt = host_threads(n);
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nt; ++t)
            pool.emplace_back(links, (uint32_t)((uint64_t)n * t / nt),
                              (uint32_t)((uint64_t)n * (t + 1) / nt));
        links(0, (uint32_t)((uint64_t)n / nt));
        for (auto& th : pool) th.join();
    }
    for (uint32_t i = 0; i < n; ++i) {
        tail[i] = i;
        pq.push(Fragment{nint_dist(p[i], p[link[i]]), i});
    }
    for (uint32_t e = 0; e + 1 < n; ++e) {
        uint32_t x, y;
        for (;;) {
            const Fragment f = pq.top();
            x = f.id;
            if (degree[x] == 2) {
                pq.pop();
                continue;
            }
            y = link[x];
            if (degree[y] < 2 && y != tail[x]) break;
            // look x's neighbour up again, without x and its fragment's far end
            link[x] = grid.nearest(p[x].x, p[x].y, x, degree[x] ? tail[x] : x);
            pq.pop();
            pq.push(Fragment{nint_dist(p[x], p[link[x]]), x});
        }
        for (const uint32_t v : {x, y}) {
            const uint32_t w = v == x ? y : x;
            if (degree[v] == 0)
                first[v] = w;
            else
                second[v] = w;
            if (++degree[v] == 2) grid.remove(v);
        }
        const uint32_t tx = tail[x];
        tail[tx] = tail[y];
        tail[tail[y]] = tx;
    }
    // list the path from city 0
    auto walk = [&](int64_t from, int64_t at, std::vector<uint32_t>& out) {
        while (at >= 0) {
            out.push_back((uint32_t)at);
            const int64_t nx = first[at] == from ? second[at] : first[at];
            from = at;
            at = nx;
        }
    };
    std::vector<uint32_t> before, after;
    walk(0, first[0], before);
    walk(0, second[0], after);
    uint32_t k = 0;
    for (auto it = before.rbegin(); it != before.rend(); ++it) route[k++] = *it;
    route[k++] = 0;
    for (const uint32_t v : after) route[k++] = v;
}

bool finite_coords(const logo_xy* c, uint32_t n) {
    for (uint32_t k = 0; k < n; ++k)
        if (!std::isfinite(c[k].x) || !std::isfinite(c[k].y)) return false;
    return true;
}

// TSPLIB header keyword of a line ("DIMENSION : 52" -> "DIMENSION"), without
// blanks; `colon` receives the position of ':' or npos.
std::string header_key(const std::string& s, size_t& colon) {
    colon = s.find(':');
    std::string key = s.substr(0, colon == std::string::npos ? s.size() : colon);
    key.erase(std::remove_if(key.begin(), key.end(), ::isspace), key.end());
    return key;
}

std::string header_value(const std::string& s, size_t colon) {
    std::string v = colon == std::string::npos ? std::string() : s.substr(colon + 1);
    v.erase(std::remove_if(v.begin(), v.end(), ::isspace), v.end());
    return v;
}

}  // namespace

namespace logo {

// k nearest other cities of every city (by squared double distance, ties to
// the lower id), written as out[v * k + j], nearest first; fewer than k
// other cities leave the remaining slots at the last one found (or v itself
// when n == 1).  A uniform grid of about two cities per cell; each query
// scans square rings of cells until k candidates are held and the next ring
// is farther than the k-th (with a relative allowance for the rounding of
// the cell arithmetic, so the lists are exact).  The boxed sweep seeds its
// bound with these pairs (any list keeps its results exact); the neighbour
// search (LOGO_SEARCH_NEIGHBOUR) takes its candidate moves from them.
void knn_grid(const logo_xy* p, uint32_t n, uint32_t k, uint32_t* out) {
    if (n == 0 || k == 0) return;
    double x0 = p[0].x, x1 = p[0].x, y0 = p[0].y, y1 = p[0].y;
    for (uint32_t v = 1; v < n; ++v) {
        x0 = std::min<double>(x0, p[v].x); x1 = std::max<double>(x1, p[v].x);
        y0 = std::min<double>(y0, p[v].y); y1 = std::max<double>(y1, p[v].y);
    }
    const double w = std::max(x1 - x0, 1e-9), h = std::max(y1 - y0, 1e-9);
    double cell = std::sqrt(w * h * 2.0 / (double)n);
    if (!(cell > 0)) cell = std::max(w, h);
    const uint32_t gw = (uint32_t)std::min<double>(4096.0, std::floor(w / cell) + 1);
    const uint32_t gh = (uint32_t)std::min<double>(4096.0, std::floor(h / cell) + 1);
    const double cw = w / gw, ch = h / gh;
    auto cx_of = [&](double x) {
        const double t = std::floor((x - x0) / cw);
        return (uint32_t)std::min<double>(gw - 1, std::max(0.0, t));
    };
    auto cy_of = [&](double y) {
        const double t = std::floor((y - y0) / ch);
        return (uint32_t)std::min<double>(gh - 1, std::max(0.0, t));
    };
    std::vector<uint32_t> start((size_t)gw * gh + 1, 0), items(n);
    std::vector<uint32_t> cellof(n);
    for (uint32_t v = 0; v < n; ++v) {
        cellof[v] = cy_of(p[v].y) * gw + cx_of(p[v].x);
        start[cellof[v] + 1]++;
    }
    for (size_t c = 0; c < (size_t)gw * gh; ++c) start[c + 1] += start[c];
    {
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (uint32_t v = 0; v < n; ++v) items[fill[cellof[v]]++] = v;
    }
    // every city's list depends on the grid alone: cities are split into
    // contiguous ranges over host threads, the lists the same for any split
    auto lists = [&](uint32_t v_lo, uint32_t v_hi) {
    std::vector<std::pair<double, uint32_t>> best;
    best.reserve(k + 1);
    for (uint32_t v = v_lo; v < v_hi; ++v) {
        const double px = p[v].x, py = p[v].y;
        const int cx = (int)cx_of(px), cy = (int)cy_of(py);
        best.clear();
        auto offer = [&](uint32_t u) {
            if (u == v) return;
            const double dx = px - (double)p[u].x, dy = py - (double)p[u].y;
            const std::pair<double, uint32_t> e(dx * dx + dy * dy, u);
            if (best.size() == k && !(e < best.back())) return;
            best.insert(std::upper_bound(best.begin(), best.end(), e), e);
            if (best.size() > k) best.pop_back();
        };
        for (int r = 0;; ++r) {
            // cells of ring r: Chebyshev distance r from (cx, cy)
            for (int yy = cy - r; yy <= cy + r; ++yy) {
                if (yy < 0 || yy >= (int)gh) continue;
                const bool edge_row = (yy == cy - r || yy == cy + r);
                for (int xx = cx - r; xx <= cx + r; xx += (edge_row ? 1 : 2 * r)) {
                    if (xx >= 0 && xx < (int)gw) {
                        const size_t c = (size_t)yy * gw + xx;
                        for (uint32_t t = start[c]; t < start[c + 1]; ++t) offer(items[t]);
                    }
                    if (r == 0) break;
                }
            }
            // every unscanned city is at least r cells away on one axis
            const double reach = r * std::min(cw, ch) * (1.0 - 1e-9);
            if (best.size() == k && reach * reach > best.back().first) break;
            if (r > (int)(gw + gh)) break;
        }
        for (uint32_t j = 0; j < k; ++j)
            out[(size_t)v * k + j] = best.empty() ? v : best[std::min<size_t>(j, best.size() - 1)].second;
    }
    };
    const unsigned nt = host_threads(n);
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t)
        pool.emplace_back(lists, (uint32_t)((uint64_t)n * t / nt),
                          (uint32_t)((uint64_t)n * (t + 1) / nt));
    lists(0, (uint32_t)((uint64_t)n / nt));
    for (auto& th : pool) th.join();
}

}  // namespace logo

extern "C" {

logo_status logo_nn_tour(const logo_xy* coords, uint32_t n, uint32_t start, uint32_t* route) {
    if (!coords || !route || n == 0 || n > LOGO_MAX_CITIES || start >= n)
        return LOGO_ERR_INVALID_ARG;
    if (!finite_coords(coords, n)) return LOGO_ERR_INVALID_ARG;
    NNGrid g(coords, n);
    // the reference searches from city 0's own point, so the first pick is
    // city 0 itself (or an earlier-id duplicate of it)
    double px = coords[start].x, py = coords[start].y;
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t id = g.nearest(px, py);
        if (id == UINT32_MAX) return LOGO_ERR_INVALID_ARG;
        route[k] = id;
        g.remove(id);
        px = coords[id].x;
        py = coords[id].y;
    }
    return LOGO_OK;
}

logo_status logo_neighbours(const logo_xy* coords, uint32_t n, uint32_t k, uint32_t* out) {
    if (!coords || !out || n == 0 || n > LOGO_MAX_CITIES || k == 0 || k > 64)
        return LOGO_ERR_INVALID_ARG;
    if (!finite_coords(coords, n)) return LOGO_ERR_INVALID_ARG;
    logo::knn_grid(coords, n, k, out);
    return LOGO_OK;
}

logo_status logo_mf_tour(const logo_xy* coords, uint32_t n, uint32_t* route) {
    if (!coords || !route || n == 0 || n > LOGO_MAX_CITIES) return LOGO_ERR_INVALID_ARG;
    if (!finite_coords(coords, n)) return LOGO_ERR_INVALID_ARG;
    mf_tour(coords, n, route);
    return LOGO_OK;
}

logo_status logo_tsplib_info(const char* path, uint32_t* n_out, int* edge_weight_type) {
    if (!path) return LOGO_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return LOGO_ERR_NOT_FOUND;
    char line[4096];
    long dim = -1;
    int ewt = LOGO_EWT_EUC_2D;  // what the reference assumes for every file
    while (std::fgets(line, sizeof line, f)) {
        const std::string s(line);
        size_t colon;
        const std::string key = header_key(s, colon);
        if (key == "NODE_COORD_SECTION" || key == "EOF") break;
        if (key == "DIMENSION" && colon != std::string::npos)
            dim = std::strtol(s.c_str() + colon + 1, nullptr, 10);
        if (key == "EDGE_WEIGHT_TYPE") {
            const std::string v = header_value(s, colon);
            ewt = v == "EUC_2D" ? LOGO_EWT_EUC_2D
                  : v == "CEIL_2D" ? LOGO_EWT_CEIL_2D
                  : v == "ATT" ? LOGO_EWT_ATT
                  : v == "GEO" ? LOGO_EWT_GEO
                  : LOGO_EWT_OTHER;
        }
    }
    std::fclose(f);
    if (dim <= 0 || (uint64_t)dim > LOGO_MAX_CITIES) return LOGO_ERR_INVALID_ARG;
    if (n_out) *n_out = (uint32_t)dim;
    if (edge_weight_type) *edge_weight_type = ewt;
    return LOGO_OK;
}

logo_status logo_read_tour(const char* path, uint32_t* route, uint32_t cap, uint32_t* n_out) {
    if (!path || !n_out) return LOGO_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return LOGO_ERR_NOT_FOUND;
    // TSPLIB .tour (header, TOUR_SECTION, ids, -1, EOF) or the reference's
    // bare list of ids; both 1-based
    std::vector<uint32_t> ids;
    long dim = -1;
    bool section = false, bad = false;
    char line[4096];
    while (std::fgets(line, sizeof line, f)) {
        const std::string s(line);
        size_t colon;
        const std::string key = header_key(s, colon);
        if (key.empty()) continue;
        if (key == "EOF" || key == "-1") break;
        if (!section && !std::isdigit((unsigned char)key[0])) {
            if (key == "TOUR_SECTION") section = true;
            if (key == "DIMENSION" && colon != std::string::npos)
                dim = std::strtol(s.c_str() + colon + 1, nullptr, 10);
            continue;
        }
        section = true;
        const char* p = line;
        char* end;
        for (;;) {
            const long v = std::strtol(p, &end, 10);
            if (end == p) break;
            if (v == -1) goto done;
            if (v < 1 || (uint64_t)v > LOGO_MAX_CITIES) {
                bad = true;
                goto done;
            }
            ids.push_back((uint32_t)(v - 1));
            p = end;
        }
    }
done:
    std::fclose(f);
    if (bad || ids.empty() || (dim > 0 && (long)ids.size() != dim)) return LOGO_ERR_INVALID_ARG;
    const uint32_t n = (uint32_t)ids.size();
    std::vector<uint8_t> seen(n, 0);
    for (const uint32_t v : ids) {
        if (v >= n || seen[v]) return LOGO_ERR_INVALID_ARG;
        seen[v] = 1;
    }
    *n_out = n;
    if (!route) return LOGO_OK;  // size query
    if (n > cap) return LOGO_ERR_INVALID_ARG;
    std::memcpy(route, ids.data(), sizeof(uint32_t) * n);
    return LOGO_OK;
}

logo_status logo_write_tour(const char* path, const uint32_t* route, uint32_t n,
                            const char* name, int tsplib_header) {
    if (!path || !route || n == 0) return LOGO_ERR_INVALID_ARG;
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t k = 0; k < n; ++k) {
        if (route[k] >= n || seen[route[k]]) return LOGO_ERR_INVALID_ARG;
        seen[route[k]] = 1;
    }
    FILE* f = std::fopen(path, "w");
    if (!f) return LOGO_ERR_NOT_FOUND;
    bool ok = true;
    if (tsplib_header)
        ok = std::fprintf(f, "NAME : %s\nTYPE : TOUR\nDIMENSION : %u\nTOUR_SECTION\n",
                          name && *name ? name : "tour", n) > 0;
    for (uint32_t k = 0; ok && k < n; ++k) ok = std::fprintf(f, "%u\n", route[k] + 1) > 0;
    if (ok && tsplib_header) ok = std::fprintf(f, "-1\nEOF\n") > 0;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? LOGO_OK : LOGO_ERR_NOT_FOUND;
}

logo_status logo_random_tour(uint32_t n, uint64_t seed, uint32_t* route) {
    if (!route || n == 0 || n > LOGO_MAX_CITIES) return LOGO_ERR_INVALID_ARG;
    // Fisher-Yates driven by SplitMix64 from the state seed + 6*C, the same
    // stream the Python generators use for start tours
    uint64_t s = seed + 6ull * 0xD1B54A32D192ED03ull;
    for (uint32_t k = 0; k < n; ++k) route[k] = k;
    for (uint32_t k = n - 1; k >= 1; --k) {
        const uint64_t hi = splitmix64(s) >> 32;
        const uint32_t j = (uint32_t)((hi * (uint64_t)(k + 1)) >> 32);
        std::swap(route[k], route[j]);
    }
    return LOGO_OK;
}

int logo_check_tour(const uint32_t* route, uint32_t n) {
    if (!route || n < 3) return 0;
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t k = 0; k < n; ++k) {
        if (route[k] >= n || seen[route[k]]) return 0;
        seen[route[k]] = 1;
    }
    return 1;
}

// TSPLIB reader.  The reference skips exactly three header lines and then
// expects "DIMENSION: n" (src/utils/tsp_loader.c:72-102), which misreads
// files with more header lines; this reader parses "KEY : value" lines until
// NODE_COORD_SECTION, then reads "id x y" triples (coordinates as float, as
// the reference does, :127-131) until EOF or a non-numeric token.
logo_status logo_read_tsplib(const char* path, logo_xy* coords, uint32_t cap, uint32_t* n_out) {
    if (!path || !n_out) return LOGO_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return LOGO_ERR_NOT_FOUND;
    char line[4096];
    long dim = -1;
    bool in_coords = false;
    while (std::fgets(line, sizeof line, f)) {
        const std::string s(line);
        size_t colon;
        const std::string key = header_key(s, colon);
        if (key == "NODE_COORD_SECTION") {
            in_coords = true;
            break;
        }
        if (key == "DIMENSION" && colon != std::string::npos)
            dim = std::strtol(s.c_str() + colon + 1, nullptr, 10);
    }
    if (!in_coords || dim <= 0 || (uint64_t)dim > LOGO_MAX_CITIES) {
        std::fclose(f);
        return LOGO_ERR_INVALID_ARG;
    }
    *n_out = (uint32_t)dim;
    if (!coords) {  // size query
        std::fclose(f);
        return LOGO_OK;
    }
    if ((uint32_t)dim > cap) {
        std::fclose(f);
        return LOGO_ERR_INVALID_ARG;
    }
    long got = 0;
    long id;
    float x, y;
    while (got < dim && std::fscanf(f, "%ld %f %f", &id, &x, &y) == 3) {
        coords[got].x = x;
        coords[got].y = y;
        ++got;
    }
    std::fclose(f);
    if (got != dim) return LOGO_ERR_INVALID_ARG;
    return LOGO_OK;
}

}  // extern "C"
