// Closed-loop load on the served form from native client threads.
//
// Each client thread owns a share of the camera streams and keeps `inflight`
// frames outstanding per stream: it submits (uslam_server_submit), waits for
// its oldest request, copies that frame's features and matches into its own
// host buffers (uslam_server_result), releases it and submits the stream's
// next frame.  Latency runs from submit until the results are in the client's
// buffers.  Prints one JSON line.
//
// usage: server_load pattern.bin frames.bin seconds inflight threads promote_every cap_per_level
//   pattern.bin: 256 x 4 int32 (the BRIEF tests)
//   frames.bin:  int32 n_streams, then per stream int32 w, h, n and n frames of w*h bytes
#include <uslam.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <fstream>
#include <mutex>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct Stream {
    int w = 0, h = 0, id = 0;
    std::vector<std::vector<uint8_t>> frames;
    long count = 0;
    int outstanding = 0;
};

struct Pending {
    uint64_t ticket;
    int stream;
    Clock::time_point t_submit;
};

// forwards through the trajectory, then backwards, and again
int walk(long count, int n) {
    if (n <= 1) return 0;
    const long period = 2L * (n - 1);
    const long k = count % period;
    return static_cast<int>(k < n ? k : period - k);
}

bool read_all(const char* path, std::vector<char>* out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    out->assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: %s pattern.bin frames.bin seconds inflight threads promote_every cap_per_level\n",
                     argv[0]);
        return 2;
    }
    const double seconds = std::atof(argv[3]);
    const int inflight = std::atoi(argv[4]);
    const int nthreads = std::atoi(argv[5]);
    const int promote_every = std::atoi(argv[6]);
    const int cap_per_level = std::atoi(argv[7]);
    std::vector<char> pat_bytes, frame_bytes;
    if (!read_all(argv[1], &pat_bytes) || pat_bytes.size() != 256 * 4 * sizeof(int32_t) ||
        !read_all(argv[2], &frame_bytes)) {
        std::fprintf(stderr, "bad input files\n");
        return 2;
    }
    size_t off = 0;
    auto take_i32 = [&](int32_t* v) {
        if (off + 4 > frame_bytes.size()) return false;
        std::copy(frame_bytes.data() + off, frame_bytes.data() + off + 4, reinterpret_cast<char*>(v));
        off += 4;
        return true;
    };
    int32_t ns = 0;
    if (!take_i32(&ns) || ns < 1) return 2;
    std::vector<Stream> streams(ns);
    int max_w = 1, max_h = 1;
    std::vector<std::pair<int, int>> sizes;
    for (auto& s : streams) {
        int32_t w, h, n;
        if (!take_i32(&w) || !take_i32(&h) || !take_i32(&n) || w < 1 || h < 1 || n < 1) return 2;
        s.w = w;
        s.h = h;
        for (int i = 0; i < n; ++i) {
            const size_t bytes = static_cast<size_t>(w) * h;
            if (off + bytes > frame_bytes.size()) return 2;
            s.frames.emplace_back(frame_bytes.begin() + off, frame_bytes.begin() + off + bytes);
            off += bytes;
        }
        max_w = std::max(max_w, w);
        max_h = std::max(max_h, h);
        if (std::find(sizes.begin(), sizes.end(), std::make_pair(s.w, s.h)) == sizes.end()) sizes.emplace_back(s.w, s.h);
    }
    frame_bytes.clear();
    frame_bytes.shrink_to_fit();

    uslam_params p{};
    p.device = 0;
    p.levels = 6;
    p.max_width = max_w;
    p.max_height = max_h;
    p.cap_per_level = cap_per_level;
    p.brief_pattern = reinterpret_cast<const int32_t*>(pat_bytes.data());
    uslam_ctx* ctx = nullptr;
    if (uslam_create(&p, &ctx) != USLAM_OK) {
        std::fprintf(stderr, "uslam_create failed\n");
        return 1;
    }
    std::vector<int> ws, hs;
    for (auto& sz : sizes) {
        ws.push_back(sz.first);
        hs.push_back(sz.second);
    }
    uslam_server_params sp{};
    sp.n_sizes = static_cast<int>(sizes.size());
    sp.widths = ws.data();
    sp.heights = hs.data();
    sp.hbm_budget_bytes = size_t(8) << 30;
    sp.max_batch = 64;
    uslam_server* srv = nullptr;
    if (uslam_server_create(ctx, &sp, &srv) != USLAM_OK) {
        std::fprintf(stderr, "server_create: %s\n", uslam_last_error(ctx));
        uslam_destroy(ctx);
        return 1;
    }
    for (auto& s : streams) {
        if (uslam_server_open_stream(srv, s.w, s.h, &s.id) != USLAM_OK) {
            std::fprintf(stderr, "open_stream: %s\n", uslam_last_error(ctx));
            return 1;
        }
    }

    const int max_feats = 6 * (cap_per_level > 0 ? cap_per_level : max_w * max_h / 250 + 1);
    std::atomic<int> failed{0};
    std::atomic<long> refused{0};
    std::mutex lat_mu;
    std::vector<double> lat;
    const auto start = Clock::now();
    const auto deadline = start + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(seconds));

    auto client = [&](int me) {
        std::vector<uslam_feature> feats(max_feats);
        std::vector<uslam_match> matches(max_feats);
        int kept[6], raw[6];
        std::vector<double> mine;
        std::deque<Pending> fifo;
        std::vector<int> own;
        for (int k = me; k < ns; k += nthreads) own.push_back(k);
        auto submit = [&](int k) {
            Stream& s = streams[k];
            const auto& img = s.frames[walk(s.count, static_cast<int>(s.frames.size()))];
            uint64_t tk = 0;
            const auto t0 = Clock::now();
            const uslam_status st =
                uslam_server_submit(srv, s.id, img.data(), s.w, s.count % promote_every == 0 ? 1 : 0, &tk);
            if (st == USLAM_CAPACITY) {
                ++refused;
                return false;
            }
            if (st != USLAM_OK) {
                ++failed;
                return false;
            }
            ++s.count;
            ++s.outstanding;
            fifo.push_back(Pending{tk, k, t0});
            return true;
        };
        bool running = true;
        while (!failed.load()) {
            running = Clock::now() < deadline;
            if (running)
                for (int k : own)
                    while (streams[k].outstanding < inflight && submit(k)) {
                    }
            if (fifo.empty()) {
                if (!running) break;
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                continue;
            }
            const Pending pd = fifo.front();
            fifo.pop_front();
            if (uslam_server_wait(srv, pd.ticket, 0) != USLAM_OK) {
                ++failed;
                break;
            }
            int nm = 0;
            double srv_ms = 0.0;
            const uslam_status st = uslam_server_result(srv, pd.ticket, feats.data(), max_feats, kept, raw,
                                                         matches.data(), max_feats, &nm, &srv_ms);
            if (st != USLAM_OK && st != USLAM_NOT_READY) {
                ++failed;
                break;
            }
            mine.push_back(std::chrono::duration<double, std::milli>(Clock::now() - pd.t_submit).count());
            uslam_server_release(srv, pd.ticket);
            --streams[pd.stream].outstanding;
        }
        std::lock_guard<std::mutex> g(lat_mu);
        lat.insert(lat.end(), mine.begin(), mine.end());
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(client, t);
    for (auto& t : th) t.join();
    const double elapsed = std::chrono::duration<double>(Clock::now() - start).count();
    uint64_t launches = 0, frames = 0;
    int max_batch_seen = 0, slots = 0;
    uslam_server_stats(srv, &launches, &frames, &max_batch_seen, &slots);
    uslam_server_destroy(srv);
    uslam_destroy(ctx);
    if (failed.load() || lat.empty()) {
        std::fprintf(stderr, "client failures: %d\n", failed.load());
        return 1;
    }
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) { return lat[std::min(lat.size() - 1, static_cast<size_t>(q * (lat.size() - 1) + 0.5))]; };
    std::printf(
        "{\"frames\": %zu, \"seconds\": %.3f, \"frames_per_s\": %.1f, \"p50_ms\": %.4f, \"p99_ms\": %.4f, "
        "\"max_ms\": %.4f, \"launches\": %llu, \"frames_per_launch\": %.3f, \"max_batch_seen\": %d, "
        "\"admission_retries\": %ld}\n",
        lat.size(), elapsed, lat.size() / elapsed, pct(0.5), pct(0.99), lat.back(),
        static_cast<unsigned long long>(launches), launches ? static_cast<double>(frames) / launches : 0.0,
        max_batch_seen, refused.load());
    return 0;
}
