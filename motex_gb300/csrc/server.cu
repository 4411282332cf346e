// Extraction server: continuous batching of extraction requests on one GPU.
//
// Requests are copied at submission and queued.  Each worker thread owns
// its own engine context (own stream and device buffers) and repeatedly
// admits the longest prefix of the queue that fits both the batch limit and
// the device-memory budget still free, runs it as one batch
// (motex_gpu_run_batch: one persistent DP launch per kernel class), and
// publishes the results.  With two or more workers a batch is admitted while
// the previous one is still on the GPU, so their device work overlaps and
// requests that arrive mid-batch are picked up as soon as a worker and
// memory free up.  Waiting is on the host only (condition variables with a
// timeout); nothing spins on the device.
#include "motex_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace
{

using Clock = std::chrono::steady_clock;

double ms_between ( Clock::time_point a, Clock::time_point b )
{
    return std::chrono::duration<double, std::milli> ( b - a ).count ();
}

struct Request
{
    uint64_t id = 0;
    std::string text;                            // all sequences back to back
    std::vector<uint32_t> lens;
    std::vector<const char *> ptrs;
    motex_params prm {};
    std::vector<uint32_t> gmin, gmax, blens, berrs;
    uint64_t footprint = 0;
    Clock::time_point t_submit, t_start, t_done;
    uint32_t batch = 0;
    int rc = MOTEX_OK;
    std::string err;
    motex_result res {};
    bool done = false;
    bool taken = false;
};

} // namespace

struct motex_server
{
    int device = 0;
    uint64_t budget = 0;
    uint32_t max_batch = 1;
    uint32_t max_queue = 0;
    std::vector<motex_ctx *> ctxs;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t in_use = 0;
    uint64_t next_id = 1;
    bool stop = false;
    motex_srv_stats stats {};
};

namespace
{

/*
 * Upper estimate of the device bytes one request keeps while it runs:
 * per input symbol the upload, codes, planes, masks and the per-position
 * filter arrays; per factor end the sort buffers, factor planes and
 * accumulators; structured requests hold per (position, gap choice)
 * accumulators and filter arrays instead.
 */
uint64_t footprint ( const Request & r )
{
    const uint64_t T = r.text.size ();
    uint64_t words = 0;
    for ( uint32_t n : r.lens )
        if ( n >= r.prm.l ) words += n - r.prm.l + 1;
    uint64_t b = 4096 + T * 18 + words * 64 + ( uint64_t ) r.lens.size () * 16;
    if ( r.prm.nb_gaps )
    {
        const uint64_t G = r.gmax[0] - r.gmin[0] + 1;
        b += T * G * 24 + T * 48;
    }
    return b;
}

void worker_loop ( motex_server * s, motex_ctx * ctx )
{
    cudaSetDevice ( s->device );
    std::unique_lock<std::mutex> lk ( s->mu );
    for ( ;; )
    {
        s->cv_work.wait ( lk, [&] { return s->stop || ! s->queue.empty (); } );
        if ( s->stop && s->queue.empty () ) return;
        // admit the longest prefix that fits the batch limit and the free memory
        std::vector<Request *> batch;
        uint64_t need = 0;
        while ( ! s->queue.empty () && batch.size () < s->max_batch )
        {
            Request * r = s->queue.front ();
            const bool fits = s->in_use + need + r->footprint <= s->budget;
            if ( ! fits && ! ( batch.empty () && s->in_use == 0 ) ) break;   // alone, it always runs
            batch.push_back ( r );
            need += r->footprint;
            s->queue.pop_front ();
        }
        if ( batch.empty () )
        {
            // memory is held by batches in flight: wait for one to finish
            s->cv_work.wait ( lk );
            continue;
        }
        s->in_use += need;
        const Clock::time_point t0 = Clock::now ();
        for ( Request * r : batch ) r->t_start = t0;
        lk.unlock ();

        std::vector<motex_job> jobs ( batch.size () );
        std::vector<motex_result> res ( batch.size () );
        for ( size_t i = 0; i < batch.size (); ++i )
            jobs[i] = motex_job { &batch[i]->prm, batch[i]->ptrs.data (), batch[i]->lens.data (),
                                  ( uint32_t ) batch[i]->lens.size () };
        int rc = motex_gpu_run_batch ( ctx, jobs.data (), ( uint32_t ) jobs.size (), res.data () );
        std::string err = rc == MOTEX_OK ? std::string () : std::string ( motex_gpu_last_error () );
        if ( rc != MOTEX_OK && batch.size () > 1 )
        {
            // isolate the failing request: run each one alone
            for ( size_t i = 0; i < batch.size (); ++i )
            {
                motex_result_free ( &res[i] );
                batch[i]->rc = motex_gpu_run_batch ( ctx, &jobs[i], 1, &res[i] );
                if ( batch[i]->rc != MOTEX_OK ) batch[i]->err = motex_gpu_last_error ();
            }
        }
        else
            for ( Request * r : batch )
            {
                r->rc = rc;
                r->err = err;
            }
        const Clock::time_point t1 = Clock::now ();

        lk.lock ();
        s->in_use -= need;
        s->stats.batches++;
        s->stats.max_batch_seen = std::max<uint32_t> ( s->stats.max_batch_seen, ( uint32_t ) batch.size () );
        for ( size_t i = 0; i < batch.size (); ++i )
        {
            Request * r = batch[i];
            r->res = res[i];
            r->t_done = t1;
            r->batch = ( uint32_t ) batch.size ();
            r->done = true;
            s->stats.completed++;
            if ( r->rc != MOTEX_OK ) s->stats.failed++;
            s->stats.cells += r->res.ref_cells;
        }
        s->cv_done.notify_all ();
        s->cv_work.notify_all ();
    }
}

} // namespace

extern "C" {

int motex_srv_create ( motex_server ** out, int device, uint64_t hbm_budget_bytes, uint32_t max_batch,
                       uint32_t workers, uint32_t max_queue )
{
    if ( ! out || max_batch == 0 || workers == 0 ) return MOTEX_EINVAL;
    *out = nullptr;
    std::unique_ptr<motex_server> s ( new motex_server () );
    s->device = device;
    s->max_batch = max_batch;
    s->max_queue = max_queue;
    if ( cudaSetDevice ( device ) != cudaSuccess ) return MOTEX_ECUDA;
    if ( hbm_budget_bytes == 0 )
    {
        size_t freeb = 0, totalb = 0;
        if ( cudaMemGetInfo ( &freeb, &totalb ) != cudaSuccess ) return MOTEX_ECUDA;
        hbm_budget_bytes = freeb / 2;             // leave room for the workers' cached buffers
    }
    s->budget = hbm_budget_bytes;
    for ( uint32_t w = 0; w < workers; ++w )
    {
        motex_ctx * c = nullptr;
        int rc = motex_ctx_create ( &c, device );
        if ( rc != MOTEX_OK )
        {
            for ( motex_ctx * x : s->ctxs ) motex_ctx_destroy ( x );
            return rc;
        }
        s->ctxs.push_back ( c );
    }
    motex_server * raw = s.get ();
    for ( motex_ctx * c : s->ctxs ) s->threads.emplace_back ( worker_loop, raw, c );
    *out = s.release ();
    return MOTEX_OK;
}

int motex_srv_submit ( motex_server * s, const motex_job * job, uint64_t * id )
{
    if ( ! s || ! job || ! job->prm || ! id || ( job->nseq && ( ! job->seqs || ! job->lens ) ) ) return MOTEX_EINVAL;
    std::unique_ptr<Request> r ( new Request () );
    size_t total = 0;
    for ( uint32_t i = 0; i < job->nseq; ++i ) total += job->lens[i];
    r->text.reserve ( total );
    r->lens.assign ( job->lens, job->lens + job->nseq );
    for ( uint32_t i = 0; i < job->nseq; ++i )
    {
        if ( job->lens[i] && ! job->seqs[i] ) return MOTEX_EINVAL;
        r->text.append ( job->seqs[i], job->lens[i] );
    }
    size_t at = 0;
    for ( uint32_t i = 0; i < job->nseq; ++i )
    {
        r->ptrs.push_back ( r->text.data () + at );
        at += job->lens[i];
    }
    r->prm = *job->prm;
    const uint32_t g = job->prm->nb_gaps;
    if ( g && ( ! job->prm->gap_min || ! job->prm->gap_max || ! job->prm->blens || ! job->prm->berrs ) ) return MOTEX_EINVAL;
    r->gmin.assign ( job->prm->gap_min, job->prm->gap_min + g );
    r->gmax.assign ( job->prm->gap_max, job->prm->gap_max + g );
    r->blens.assign ( job->prm->blens, job->prm->blens + g );
    r->berrs.assign ( job->prm->berrs, job->prm->berrs + g );
    r->prm.gap_min = r->gmin.data ();
    r->prm.gap_max = r->gmax.data ();
    r->prm.blens = r->blens.data ();
    r->prm.berrs = r->berrs.data ();
    if ( g && r->gmax[0] < r->gmin[0] ) return MOTEX_EINVAL;
    r->footprint = footprint ( *r );
    std::lock_guard<std::mutex> lk ( s->mu );
    if ( s->stop ) return MOTEX_EBUSY;
    if ( r->footprint > s->budget ) return MOTEX_ENOMEM;        // could never be admitted
    if ( s->max_queue && s->queue.size () >= s->max_queue ) return MOTEX_EBUSY;
    r->id = s->next_id++;
    r->t_submit = Clock::now ();
    *id = r->id;
    s->queue.push_back ( r.get () );
    s->reqs[r->id] = std::move ( r );
    s->stats.submitted++;
    s->cv_work.notify_one ();
    return MOTEX_OK;
}

int motex_srv_wait ( motex_server * s, uint64_t id, int timeout_ms, motex_result * out, motex_srv_timing * timing )
{
    if ( ! s || ! out ) return MOTEX_EINVAL;
    std::unique_lock<std::mutex> lk ( s->mu );
    auto it = s->reqs.find ( id );
    if ( it == s->reqs.end () || it->second->taken ) return MOTEX_ENOTFOUND;
    Request * r = it->second.get ();
    auto ready = [&] { return r->done; };
    if ( timeout_ms < 0 ) s->cv_done.wait ( lk, ready );
    else if ( ! s->cv_done.wait_for ( lk, std::chrono::milliseconds ( timeout_ms ), ready ) ) return MOTEX_ETIMEOUT;
    *out = r->res;                                // ownership of the motif array passes to the caller
    r->res.motifs = nullptr;
    if ( timing )
    {
        timing->queue_ms = ms_between ( r->t_submit, r->t_start );
        timing->run_ms = ms_between ( r->t_start, r->t_done );
        timing->latency_ms = ms_between ( r->t_submit, r->t_done );
        timing->batch_size = r->batch;
    }
    const int rc = r->rc;
    s->reqs.erase ( it );
    return rc;
}

int motex_srv_stats_get ( motex_server * s, motex_srv_stats * out )
{
    if ( ! s || ! out ) return MOTEX_EINVAL;
    std::lock_guard<std::mutex> lk ( s->mu );
    *out = s->stats;
    out->queued = ( uint32_t ) s->queue.size ();
    out->in_use_bytes = s->in_use;
    out->budget_bytes = s->budget;
    return MOTEX_OK;
}

int motex_srv_destroy ( motex_server * s )
{
    if ( ! s ) return MOTEX_OK;
    {
        std::lock_guard<std::mutex> lk ( s->mu );
        s->stop = true;
        s->cv_work.notify_all ();
    }
    for ( auto & t : s->threads ) t.join ();      // workers drain the queue first
    for ( motex_ctx * c : s->ctxs ) motex_ctx_destroy ( c );
    for ( auto & kv : s->reqs ) motex_result_free ( &kv.second->res );
    delete s;
    return MOTEX_OK;
}

} // extern "C"
