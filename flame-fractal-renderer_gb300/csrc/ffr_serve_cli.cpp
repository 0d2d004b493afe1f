// ffr-serve: the serving loop (ffr_server_*) behind the framing of
// include/ffr_wire.h, for remote clients.  No reference counterpart (the
// reference renders one flame per ffr-buf process).
//
//   ffr-serve --port P [--host 127.0.0.1]   TCP, one thread per connection;
//                                           all connections share one server
//                                           (a job submitted on one can be
//                                           waited for on another)
//   ffr-serve --stdio                       one client on stdin / stdout
// Server options: --device N, --precision fp32|fp64, --settle N (53),
// --traj-len N (4096), --hbm-budget BYTES (0 = free memory - 2 GiB),
// --max-active N (256), --timeout-ms N (0).
//
// With --port 0 the kernel picks a free port; the chosen port is printed on
// stderr as "listening on 127.0.0.1:<port>".  A SHUTDOWN request stops the
// accept loop, closes the other connections, destroys the server (cancelling
// what is still queued or running) and exits 0.
#include <arpa/inet.h>
#include <netinet/in.h>
#include <poll.h>
#include <sys/socket.h>
#include <unistd.h>

#include <atomic>
#include <cerrno>
#include <csignal>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ffr_gpu.h"
#include "ffr_wire.h"

namespace {

constexpr uint64_t kMaxJson = 64ull << 20;
constexpr uint64_t kMaxInit = 1ull << 40;

std::atomic<bool> g_stop{false};
std::mutex g_conn_mu;
std::vector<int> g_conns;

[[noreturn]] void die(const std::string& m)
{
    std::cerr << "ERROR: " << m << std::endl;
    std::exit(1);
}

bool read_full(int fd, void* p, size_t n)
{
    char* c = static_cast<char*>(p);
    while (n)
    {
        const ssize_t k = ::read(fd, c, n);
        if (k < 0 && errno == EINTR)
            continue;
        if (k <= 0)
            return false;
        c += k;
        n -= (size_t)k;
    }
    return true;
}

bool write_full(int fd, const void* p, size_t n)
{
    const char* c = static_cast<const char*>(p);
    while (n)
    {
        const ssize_t k = ::write(fd, c, n);
        if (k < 0 && errno == EINTR)
            continue;
        if (k <= 0)
            return false;
        c += k;
        n -= (size_t)k;
    }
    return true;
}

bool reply(int fd, ffr_status st, uint64_t job, const ffr_job_info* info, const void* payload,
           uint64_t len)
{
    ffr_wire_response r;
    std::memset(&r, 0, sizeof r);
    std::memcpy(r.magic, "FFRR", 4);
    r.status = (uint32_t)st;
    r.job = job;
    if (info)
    {
        r.state = (uint32_t)info->state;
        r.job_status = (uint32_t)info->status;
        r.samples = info->samples;
        r.buffer_bytes = info->buffer_bytes;
        r.parent = info->parent;
        r.submit_ns = info->submit_ns;
        r.admit_ns = info->admit_ns;
        r.done_ns = info->done_ns;
    }
    r.payload_len = len;
    return write_full(fd, &r, sizeof r) && (len == 0 || write_full(fd, payload, len));
}

bool reply_error(int fd, ffr_server* srv, ffr_status st, uint64_t job)
{
    const std::string m = ffr_server_last_error(srv);
    return reply(fd, st, job, nullptr, m.data(), m.size());
}

// Requests of one connection, in turn, until it closes or asks to shut down.
void serve(ffr_server* srv, int in_fd, int out_fd)
{
    std::vector<char> json;
    std::vector<unsigned char> init, buf;
    for (;;)
    {
        ffr_wire_request rq;
        if (!read_full(in_fd, &rq, sizeof rq))
            return;
        if (std::memcmp(rq.magic, "FFRQ", 4) != 0 || rq.version != FFR_WIRE_VERSION
                || rq.json_len > kMaxJson || rq.init_len > kMaxInit)
        {
            const std::string m = "bad request frame";
            reply(out_fd, FFR_ERR_ARG, 0, nullptr, m.data(), m.size());
            return;
        }
        json.resize(rq.json_len);
        init.resize(rq.init_len);
        if ((rq.json_len && !read_full(in_fd, json.data(), json.size()))
                || (rq.init_len && !read_full(in_fd, init.data(), init.size())))
            return;
        ffr_job_info info;
        std::memset(&info, 0, sizeof info);
        uint64_t job = rq.job;
        ffr_status st = FFR_OK;
        bool ok = true;
        switch (rq.op)
        {
        case FFR_WIRE_SUBMIT:
        case FFR_WIRE_CONTINUE:
            st = rq.op == FFR_WIRE_SUBMIT
                ? ffr_server_submit(srv, json.data(), json.size(),
                                    rq.init_len ? init.data() : nullptr, init.size(), rq.samples,
                                    rq.seed, rq.bad_limit, &job)
                : ffr_server_continue(srv, rq.job, rq.samples, rq.seed, rq.bad_limit, &job);
            if (st == FFR_OK)
                ffr_server_poll(srv, job, &info);
            ok = st == FFR_OK ? reply(out_fd, st, job, &info, nullptr, 0)
                              : reply_error(out_fd, srv, st, job);
            break;
        case FFR_WIRE_WAIT:
        case FFR_WIRE_READ:
        case FFR_WIRE_POLL:
        {
            if (rq.op == FFR_WIRE_WAIT)
            {
                // wait in slices so a shutdown is never held up by a long job
                uint64_t waited = 0;
                for (;;)
                {
                    uint64_t slice = 200;
                    if (rq.timeout_ms && rq.timeout_ms - waited < slice)
                        slice = rq.timeout_ms - waited;
                    st = ffr_server_wait(srv, job, slice ? slice : 1, &info);
                    waited += slice;
                    if (st != FFR_ERR_TIMEOUT || g_stop
                            || (rq.timeout_ms && waited >= rq.timeout_ms))
                        break;
                }
            }
            else
                st = ffr_server_poll(srv, job, &info);
            const bool want = rq.op == FFR_WIRE_READ
                || (rq.op == FFR_WIRE_WAIT && (rq.flags & FFR_WIRE_WITH_BUFFER));
            if (st == FFR_OK && want)
            {
                buf.resize(info.buffer_bytes);
                st = ffr_server_read(srv, job, buf.data(), buf.size());
            }
            if (st != FFR_OK)
                ok = reply_error(out_fd, srv, st, job);
            else
                ok = reply(out_fd, st, job, &info, want ? buf.data() : nullptr,
                           want ? buf.size() : 0);
            break;
        }
        case FFR_WIRE_CANCEL:
        case FFR_WIRE_RELEASE:
            st = rq.op == FFR_WIRE_CANCEL ? ffr_server_cancel(srv, job)
                                          : ffr_server_release(srv, job);
            ok = st == FFR_OK ? reply(out_fd, st, job, nullptr, nullptr, 0)
                              : reply_error(out_fd, srv, st, job);
            break;
        case FFR_WIRE_SHUTDOWN:
            g_stop = true;
            reply(out_fd, FFR_OK, 0, nullptr, nullptr, 0);
            return;
        default:
        {
            const std::string m = "unknown request op " + std::to_string(rq.op);
            ok = reply(out_fd, FFR_ERR_ARG, job, nullptr, m.data(), m.size());
        }
        }
        if (!ok)
            return;
    }
}

uint64_t to_u64(const std::string& v, const std::string& opt)
{
    char* end = nullptr;
    errno = 0;
    const unsigned long long x = std::strtoull(v.c_str(), &end, 10);
    if (v.empty() || v[0] == '-' || errno || *end)
        die("the argument ('" + v + "') for option '" + opt + "' is invalid");
    return x;
}

} // namespace

int main(int argc, char** argv)
{
    ffr_server_opts o;
    ffr_server_default_opts(&o);
    bool stdio = false, have_port = false;
    uint64_t port = 0;
    std::string host = "127.0.0.1";
    for (int k = 1; k < argc; ++k)
    {
        const std::string t = argv[k];
        auto val = [&]() -> std::string {
            if (k + 1 >= argc)
                die("the required argument for option '" + t + "' is missing");
            return argv[++k];
        };
        if (t == "--stdio") stdio = true;
        else if (t == "--port") { port = to_u64(val(), t); have_port = true; }
        else if (t == "--host") host = val();
        else if (t == "--device") o.device = (int32_t)to_u64(val(), t);
        else if (t == "--precision")
        {
            const std::string p = val();
            if (p == "fp32") o.precision = FFR_FP32;
            else if (p == "fp64") o.precision = FFR_FP64;
            else die("--precision must be fp64 or fp32");
        }
        else if (t == "--settle") o.settle = to_u64(val(), t);
        else if (t == "--traj-len") o.traj_len = to_u64(val(), t);
        else if (t == "--hbm-budget") o.hbm_budget = to_u64(val(), t);
        else if (t == "--max-active") o.max_active = to_u64(val(), t);
        else if (t == "--timeout-ms") o.timeout_ms = to_u64(val(), t);
        else if (t == "-h" || t == "--help")
        {
            std::cerr << "usage: ffr-serve (--port P [--host H] | --stdio) [--device N] "
                         "[--precision fp32|fp64] [--settle N] [--traj-len N] "
                         "[--hbm-budget BYTES] [--max-active N] [--timeout-ms N]\n";
            return 1;
        }
        else
            die("unrecognised option '" + t + "'");
    }
    if (stdio == have_port)
        die("choose exactly one of --port and --stdio");
    if (port > 65535)
        die("port out of range");
    std::signal(SIGPIPE, SIG_IGN);
    ffr_server* srv = nullptr;
    if (ffr_server_create(&o, &srv) != FFR_OK)
        die(ffr_last_error(nullptr));
    if (stdio)
    {
        serve(srv, 0, 1);
        ffr_server_destroy(srv);
        return 0;
    }
    const int ls = ::socket(AF_INET, SOCK_STREAM, 0);
    if (ls < 0)
        die("socket: " + std::string(std::strerror(errno)));
    const int one = 1;
    ::setsockopt(ls, SOL_SOCKET, SO_REUSEADDR, &one, sizeof one);
    sockaddr_in addr;
    std::memset(&addr, 0, sizeof addr);
    addr.sin_family = AF_INET;
    addr.sin_port = htons((uint16_t)port);
    if (::inet_pton(AF_INET, host.c_str(), &addr.sin_addr) != 1)
        die("bad --host " + host);
    if (::bind(ls, reinterpret_cast<sockaddr*>(&addr), sizeof addr) != 0 || ::listen(ls, 64) != 0)
        die("bind/listen: " + std::string(std::strerror(errno)));
    socklen_t alen = sizeof addr;
    ::getsockname(ls, reinterpret_cast<sockaddr*>(&addr), &alen);
    std::cerr << "listening on " << host << ":" << ntohs(addr.sin_port) << std::endl;
    std::vector<std::thread> threads;
    while (!g_stop)
    {
        pollfd pf{ls, POLLIN, 0};
        if (::poll(&pf, 1, 200) <= 0)
            continue;
        const int c = ::accept(ls, nullptr, nullptr);
        if (c < 0)
            continue;
        {
            std::lock_guard<std::mutex> lk(g_conn_mu);
            g_conns.push_back(c);
        }
        threads.emplace_back([srv, c] { serve(srv, c, c); });
    }
    ::close(ls);
    {
        // unblock connections still waiting for a request
        std::lock_guard<std::mutex> lk(g_conn_mu);
        for (int c : g_conns)
            ::shutdown(c, SHUT_RDWR);
    }
    for (auto& t : threads)
        t.join();
    for (int c : g_conns)
        ::close(c);
    ffr_server_destroy(srv);
    return 0;
}
