// Serving layer: continuous admission of independent FLIP simulations on one GPU under a
// device-memory budget (include/bora_serve.h). Host code only: a scheduler thread admits
// queued requests as slots and memory free up and sets up each one's bora_flip handle; a
// stepper thread advances all running requests together, one bora_flip_step_batch per
// round (the pressure solve's kernels launched once for all of them), taking newly set-up
// requests in between rounds; a finisher thread orders finished requests' particles by id,
// so neither set-up nor result handling holds up a round.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bora_serve.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request
{
    uint64_t id = 0;
    bora_grid_desc grid{};
    bora_flip_params params{};
    std::vector<float> pos, vel;  // input particles; the results after the run
    std::vector<int32_t> ids;
    std::vector<float> boxes;
    int nboxes = 0;
    float band = 0.f;
    int space = BORA_SPACE_VOXEL, steps = 0;
    float dt = 0.f;
    int state = BORA_REQ_QUEUED, status = BORA_OK, steps_done = 0;
    bora_flip_handle h = nullptr;  // from set-up until the stepper has read the results back
    uint64_t nparticles = 0, estimate = 0, device_bytes = 0;
    Clock::time_point t_submit, t_admit, t_done;
    std::vector<float> step_ms;
};

double seconds( Clock::time_point a, Clock::time_point b ) { return std::chrono::duration<double>( b - a ).count(); }

// Nearest-rank percentile of a sample (q in [0, 1]); 0 for an empty sample.
double percentile( std::vector<float> v, double q )
{
    if( v.empty() ) return 0.0;
    std::sort( v.begin(), v.end() );
    const size_t k = std::min( v.size() - 1, (size_t)( q * (double)( v.size() - 1 ) + 0.5 ) );
    return v[k];
}

}  // namespace

struct bora_server
{
    bora_serve_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv;  // any state change: submit, finish, stop
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_id = 1;
    int running = 0, running_peak = 0;
    uint64_t reserved = 0, reserved_peak = 0;
    uint64_t submitted = 0, admitted = 0, done = 0, failed = 0, particle_steps = 0, steps = 0;
    std::vector<float> step_ms;  // every step of every finished request
    bool stop = false;
    std::thread scheduler, stepper, finisher;
    std::vector<Request*> starting;  // set up, not yet taken by the stepper
    struct Finished
    {
        Request* r;
        std::vector<float> pos, vel;
        std::vector<int32_t> ids;
        uint64_t psteps;
        int status;
    };
    std::deque<Finished> finishing;  // read back, waiting for the finisher
    bool stepper_done = false;

    void schedule();
    void step_loop();
    void finish_loop();
    void finish( Request* r, int status, bool ok );
    void finish_locked( Request* r, int status, bool ok );
};

void bora_server::finish( Request* r, int status, bool ok )
{
    std::lock_guard<std::mutex> lk( mu );
    finish_locked( r, status, ok );
}

void bora_server::finish_locked( Request* r, int status, bool ok )
{
    r->state = ok ? BORA_REQ_DONE : BORA_REQ_FAILED;
    r->status = status;
    r->t_done = Clock::now();
    --running;
    reserved -= r->estimate;
    if( ok )
    {
        ++done;
        steps += (uint64_t)r->steps_done;
        step_ms.insert( step_ms.end(), r->step_ms.begin(), r->step_ms.end() );
    }
    else
    {
        ++failed;
    }
    cv.notify_all();
}

namespace {

// A running request: its handle and what it has done so far.
struct Live
{
    Request* r = nullptr;
    bora_flip_handle h = nullptr;
    uint64_t psteps = 0, peak = 0;
};

// Set up a request's simulation; BORA_OK or the failing call's status.
int start_request( Request* r, bora_flip_handle* out )
{
    bora_flip_handle h = nullptr;
    int st = bora_flip_create( &r->grid, &r->params, &h );
    if( st == BORA_OK && r->nboxes > 0 ) st = bora_flip_set_colliders( h, r->boxes.data(), r->nboxes, r->band );
    if( st == BORA_OK ) st = bora_flip_set_particles( h, r->pos.data(), r->vel.data(), r->pos.size() / 3, r->space );
    if( st != BORA_OK && h ) { bora_flip_destroy( h ); h = nullptr; }
    *out = h;
    return st;
}

// The final particles as the device holds them (any order).
int read_back( bora_flip_handle h, int space, std::vector<float>& pos, std::vector<float>& vel, std::vector<int32_t>& ids )
{
    size_t n = 0;
    int st = bora_flip_num_particles( h, &n );
    if( st != BORA_OK ) return st;
    pos.resize( n * 3 );
    vel.resize( n * 3 );
    ids.resize( n );
    size_t got = 0;
    st = bora_flip_get_particles( h, pos.data(), vel.data(), nullptr, ids.data(), n, &got, space );
    pos.resize( got * 3 );
    vel.resize( got * 3 );
    ids.resize( got );
    return st;
}

}  // namespace

// Results in ascending id order (the result does not depend on the device order).
void bora_server::finish_loop()
{
    for( ;; )
    {
        Finished f;
        {
            std::unique_lock<std::mutex> lk( mu );
            cv.wait( lk, [&] { return !finishing.empty() || stepper_done; } );
            if( finishing.empty() ) return;
            f = std::move( finishing.front() );
            finishing.pop_front();
        }
        const size_t got = f.ids.size();
        std::vector<size_t> ord( got );
        for( size_t i = 0; i < got; ++i ) ord[i] = i;
        std::sort( ord.begin(), ord.end(), [&]( size_t a, size_t b ) { return f.ids[a] < f.ids[b]; } );
        std::vector<float> p2( got * 3 ), v2( got * 3 );
        std::vector<int32_t> i2( got );
        for( size_t i = 0; i < got; ++i )
        {
            std::memcpy( &p2[3 * i], &f.pos[3 * ord[i]], 12 );
            std::memcpy( &v2[3 * i], &f.vel[3 * ord[i]], 12 );
            i2[i] = f.ids[ord[i]];
        }
        std::lock_guard<std::mutex> lk( mu );
        Request* r = f.r;
        if( f.status == BORA_OK )
        {
            r->pos.swap( p2 );
            r->vel.swap( v2 );
            r->ids.swap( i2 );
            r->nparticles = r->ids.size();
            particle_steps += f.psteps;
        }
        finish_locked( r, f.status, f.status == BORA_OK );
    }
}

void bora_server::step_loop()
{
    cudaSetDevice( device );
    std::vector<Live> live;
    for( ;; )
    {
        std::vector<Request*> fresh;
        bool stopping;
        {
            std::unique_lock<std::mutex> lk( mu );
            cv.wait( lk, [&] { return stop || !starting.empty() || !live.empty(); } );
            fresh.swap( starting );
            stopping = stop;
        }
        if( stopping )  // running requests are abandoned
        {
            for( Request* r : fresh )
            {
                bora_flip_destroy( r->h );
                r->h = nullptr;
                finish( r, BORA_ERR_CAPACITY, false );
            }
            for( Live& l : live )
            {
                bora_flip_destroy( l.h );
                finish( l.r, BORA_ERR_CAPACITY, false );
            }
            std::lock_guard<std::mutex> lk( mu );
            stepper_done = true;
            cv.notify_all();
            return;
        }
        for( Request* r : fresh )
        {
            Live l;
            l.r = r;
            l.h = r->h;
            live.push_back( l );
        }
        if( live.empty() ) continue;
        // one round: every running request with steps left advances one step; requests of
        // equal dt share a batched step
        std::vector<char> taken( live.size(), 0 ), bad( live.size(), 0 );
        for( size_t a = 0; a < live.size(); ++a )
            if( live[a].r->steps_done >= live[a].r->steps ) taken[a] = 1;  // finished (or zero steps)
        for( size_t a = 0; a < live.size(); ++a )
        {
            if( taken[a] ) continue;
            std::vector<size_t> grp;
            for( size_t b = a; b < live.size(); ++b )
                if( !taken[b] && live[b].r->dt == live[a].r->dt ) { grp.push_back( b ); taken[b] = 1; }
            std::vector<bora_flip_handle> hs( grp.size() );
            std::vector<size_t> n0( grp.size() );
            for( size_t q = 0; q < grp.size(); ++q )
            {
                hs[q] = live[grp[q]].h;
                bora_flip_num_particles( hs[q], &n0[q] );
            }
            std::vector<int> st( grp.size(), BORA_OK );
            const Clock::time_point t0 = Clock::now();
            const int bst = bora_flip_step_batch( hs.data(), (int)hs.size(), live[a].r->dt, st.data() );
            const float ms = (float)( 1e3 * seconds( t0, Clock::now() ) );
            for( size_t q = 0; q < grp.size(); ++q )
            {
                Live& l = live[grp[q]];
                const int s = bst < 0 ? bst : st[q];
                if( s < 0 ) { bad[grp[q]] = 1; std::lock_guard<std::mutex> lk( mu ); l.r->status = s; continue; }
                l.psteps += n0[q];
                bora_flip_stats fs{};
                bora_flip_get_stats( l.h, &fs );
                l.peak = std::max<uint64_t>( l.peak, fs.device_bytes );
                std::lock_guard<std::mutex> lk( mu );
                l.r->step_ms.push_back( ms );
                l.r->steps_done += 1;
                l.r->nparticles = fs.num_particles;
                l.r->device_bytes = l.peak;
            }
        }
        // retire finished and failed requests
        std::vector<Live> keep;
        for( size_t q = 0; q < live.size(); ++q )
        {
            Live& l = live[q];
            if( bad[q] )
            {
                bora_flip_destroy( l.h );
                finish( l.r, l.r->status, false );
                continue;
            }
            if( l.r->steps_done < l.r->steps ) { keep.push_back( l ); continue; }
            Finished f;
            f.r = l.r;
            f.psteps = l.psteps;
            f.status = read_back( l.h, l.r->space, f.pos, f.vel, f.ids );
            bora_flip_destroy( l.h );
            std::lock_guard<std::mutex> lk( mu );
            l.r->h = nullptr;
            finishing.push_back( std::move( f ) );
            cv.notify_all();
        }
        live.swap( keep );
    }
}

void bora_server::schedule()
{
    cudaSetDevice( device );
    std::unique_lock<std::mutex> lk( mu );
    for( ;; )
    {
        cv.wait( lk, [&] {
            if( stop ) return true;
            if( queue.empty() ) return false;
            const Request* r = reqs[queue.front()].get();
            return r->estimate > cfg.hbm_budget_bytes ||
                   ( running < cfg.max_running && reserved + r->estimate <= cfg.hbm_budget_bytes );
        } );
        if( stop ) break;
        Request* r = reqs[queue.front()].get();
        queue.pop_front();
        if( r->estimate > cfg.hbm_budget_bytes )  // can never run under this budget
        {
            r->state = BORA_REQ_FAILED;
            r->status = BORA_ERR_OUT_OF_MEMORY;
            r->t_admit = r->t_done = Clock::now();
            ++failed;
            cv.notify_all();
            continue;
        }
        r->state = BORA_REQ_RUNNING;
        r->t_admit = Clock::now();
        ++running;
        ++admitted;
        reserved += r->estimate;
        running_peak = std::max( running_peak, running );
        reserved_peak = std::max( reserved_peak, reserved );
        // the request's simulation is set up here, outside the lock, while rounds go on
        lk.unlock();
        bora_flip_handle h = nullptr;
        const int st = start_request( r, &h );
        lk.lock();
        if( st == BORA_OK && stop ) { bora_flip_destroy( h ); h = nullptr; }
        if( st != BORA_OK || stop )
        {
            finish_locked( r, st != BORA_OK ? st : BORA_ERR_CAPACITY, false );
            continue;
        }
        r->h = h;
        starting.push_back( r );
        cv.notify_all();
    }
    // stopping: queued requests are dropped
    while( !queue.empty() )
    {
        Request* r = reqs[queue.front()].get();
        queue.pop_front();
        r->state = BORA_REQ_FAILED;
        r->status = BORA_ERR_CAPACITY;
        ++failed;
    }
    cv.notify_all();
}

extern "C" {

uint64_t bora_serve_estimate_bytes( const bora_grid_desc* grid, size_t n, int solver )
{
    if( !grid ) return 0;
    // particles: two 7-array buffers, adjacency, sort keys and index, live flags, staging
    const uint64_t per_particle = 2 * 28 + 4 + 12 + 4 + 24;
    // cells of active tiles: about three times the fluid cells (8 particles per cell)
    // including the air margin; fields, flags, stencil codes, solver vectors, sort counts,
    // plus the multigrid levels for the mixed form
    const uint64_t cells = std::max<uint64_t>( 512, 3 * (uint64_t)n / 8 );
    const uint64_t per_cell = 4 * 9 + 1 + 2 + 4 + 8 + 4 * 7 + 8 + 8 + ( solver == BORA_SOLVER_MIXED ? 12 : 0 );
    // virtual tile tables: activation flag (1 B), activation, its scan, the slot table and the
    // previous step's slot table (4 B each)
    const uint64_t tiles = (uint64_t)( ( grid->nx + 8 ) / 8 + 1 ) * ( ( grid->ny + 8 ) / 8 + 1 ) * ( ( grid->nz + 8 ) / 8 + 1 );
    // geometric buffer growth keeps up to 1.5x slack
    return ( 3 * ( (uint64_t)n * per_particle + cells * per_cell ) ) / 2 + tiles * 20 + ( 16ull << 20 );
}

int bora_serve_default_config( bora_serve_config* out )
{
    if( !out ) return BORA_ERR_INVALID_ARG;
    std::memset( out, 0, sizeof( *out ) );
    out->hbm_budget_bytes = 120ull * 1000 * 1000 * 1000;
    out->max_running = 64;
    return BORA_OK;
}

int bora_serve_create( const bora_serve_config* cfg, bora_serve_handle* out )
{
    if( !cfg || !out || cfg->max_running <= 0 || cfg->hbm_budget_bytes == 0 ) return BORA_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if( cudaGetDeviceCount( &ndev ) != cudaSuccess || ndev <= 0 )
    {
        cudaGetLastError();
        return BORA_ERR_NO_DEVICE;
    }
    bora_server* s = new( std::nothrow ) bora_server;
    if( !s ) return BORA_ERR_OUT_OF_MEMORY;
    s->cfg = *cfg;
    cudaGetDevice( &s->device );
    s->scheduler = std::thread( [s] { s->schedule(); } );
    s->stepper = std::thread( [s] { s->step_loop(); } );
    s->finisher = std::thread( [s] { s->finish_loop(); } );
    *out = s;
    return BORA_OK;
}

int bora_serve_destroy( bora_serve_handle s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk( s->mu );
        s->stop = true;
    }
    s->cv.notify_all();
    if( s->scheduler.joinable() ) s->scheduler.join();
    if( s->stepper.joinable() ) s->stepper.join();
    if( s->finisher.joinable() ) s->finisher.join();
    delete s;
    return BORA_OK;
}

int bora_serve_submit( bora_serve_handle s, const bora_grid_desc* grid, const bora_flip_params* params, const float* pos,
                       const float* vel, size_t n, int space, int steps, float dt, uint64_t* request_id )
{
    if( !s || !grid || !params || !request_id || ( n > 0 && !pos ) || steps < 0 || !( dt > 0.f ) )
        return BORA_ERR_INVALID_ARG;
    if( space != BORA_SPACE_WORLD && space != BORA_SPACE_VOXEL ) return BORA_ERR_INVALID_ARG;
    std::unique_ptr<Request> r( new( std::nothrow ) Request );
    if( !r ) return BORA_ERR_OUT_OF_MEMORY;
    r->grid = *grid;
    r->params = *params;
    r->pos.assign( pos, pos + 3 * n );
    if( vel ) r->vel.assign( vel, vel + 3 * n );
    else r->vel.assign( 3 * n, 0.f );
    r->space = space;
    r->steps = steps;
    r->dt = dt;
    r->nparticles = n;
    r->estimate = bora_serve_estimate_bytes( grid, n, params->solver );
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk( s->mu );
    if( s->stop ) return BORA_ERR_INVALID_ARG;
    r->id = s->next_id++;
    *request_id = r->id;
    s->queue.push_back( r->id );
    s->reqs.emplace( r->id, std::move( r ) );
    ++s->submitted;
    s->cv.notify_all();
    return BORA_OK;
}

int bora_serve_set_colliders( bora_serve_handle s, uint64_t id, const float* boxes, int count, float band )
{
    if( !s || count < 0 || ( count > 0 && !boxes ) ) return BORA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk( s->mu );
    auto it = s->reqs.find( id );
    if( it == s->reqs.end() || it->second->state != BORA_REQ_QUEUED ) return BORA_ERR_INVALID_ARG;
    Request* r = it->second.get();
    r->boxes.assign( boxes, boxes + 9 * count );
    r->nboxes = count;
    r->band = band;
    return BORA_OK;
}

int bora_serve_poll( bora_serve_handle s, uint64_t id, bora_serve_request_status* o )
{
    if( !s || !o ) return BORA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk( s->mu );
    auto it = s->reqs.find( id );
    if( it == s->reqs.end() ) return BORA_ERR_INVALID_ARG;
    const Request* r = it->second.get();
    std::memset( o, 0, sizeof( *o ) );
    o->state = r->state;
    o->status = r->status;
    o->steps_total = r->steps;
    o->steps_done = r->steps_done;
    o->num_particles = r->nparticles;
    o->estimate_bytes = r->estimate;
    o->device_bytes = r->device_bytes;
    const Clock::time_point now = Clock::now();
    if( r->state == BORA_REQ_QUEUED ) o->queued_s = seconds( r->t_submit, now );
    else
    {
        o->queued_s = seconds( r->t_submit, r->t_admit );
        o->run_s = seconds( r->t_admit, r->state == BORA_REQ_RUNNING ? now : r->t_done );
    }
    o->step_ms_p50 = percentile( r->step_ms, 0.5 );
    o->step_ms_p99 = percentile( r->step_ms, 0.99 );
    o->step_ms_max = r->step_ms.empty() ? 0.0 : *std::max_element( r->step_ms.begin(), r->step_ms.end() );
    return BORA_OK;
}

int bora_serve_wait( bora_serve_handle s, uint64_t id, double timeout_s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk( s->mu );
    auto it = s->reqs.find( id );
    if( it == s->reqs.end() ) return BORA_ERR_INVALID_ARG;
    Request* r = it->second.get();
    auto finished = [&] { return r->state == BORA_REQ_DONE || r->state == BORA_REQ_FAILED; };
    if( timeout_s < 0.0 ) s->cv.wait( lk, finished );
    else if( !s->cv.wait_for( lk, std::chrono::duration<double>( timeout_s ), finished ) ) return BORA_WARN_TIMEOUT;
    return BORA_OK;
}

int bora_serve_result( bora_serve_handle s, uint64_t id, float* pos, float* vel, int32_t* ids, size_t cap, size_t* n )
{
    if( !s || !n ) return BORA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk( s->mu );
    auto it = s->reqs.find( id );
    if( it == s->reqs.end() || it->second->state != BORA_REQ_DONE ) return BORA_ERR_INVALID_ARG;
    const Request* r = it->second.get();
    const size_t m = r->ids.size();
    *n = m;
    if( m > cap ) return BORA_ERR_CAPACITY;
    if( pos ) std::memcpy( pos, r->pos.data(), m * 12 );
    if( vel ) std::memcpy( vel, r->vel.data(), m * 12 );
    if( ids ) std::memcpy( ids, r->ids.data(), m * 4 );
    return BORA_OK;
}

int bora_serve_release( bora_serve_handle s, uint64_t id )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk( s->mu );
    auto it = s->reqs.find( id );
    if( it == s->reqs.end() ) return BORA_ERR_INVALID_ARG;
    Request* r = it->second.get();
    if( r->state != BORA_REQ_DONE && r->state != BORA_REQ_FAILED ) return BORA_ERR_INVALID_ARG;
    s->reqs.erase( it );
    return BORA_OK;
}

int bora_serve_drain( bora_serve_handle s )
{
    if( !s ) return BORA_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk( s->mu );
    s->cv.wait( lk, [&] { return s->queue.empty() && s->running == 0; } );
    return BORA_OK;
}

int bora_serve_get_stats( bora_serve_handle s, bora_serve_stats* o )
{
    if( !s || !o ) return BORA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk( s->mu );
    std::memset( o, 0, sizeof( *o ) );
    o->submitted = s->submitted;
    o->admitted = s->admitted;
    o->done = s->done;
    o->failed = s->failed;
    o->queued = (int)s->queue.size();
    o->running = s->running;
    o->bytes_reserved = s->reserved;
    o->bytes_reserved_peak = s->reserved_peak;
    o->running_peak = s->running_peak;
    o->particle_steps = s->particle_steps;
    o->steps = s->steps;
    o->step_ms_p50 = percentile( s->step_ms, 0.5 );
    o->step_ms_p99 = percentile( s->step_ms, 0.99 );
    o->step_ms_max = s->step_ms.empty() ? 0.0 : *std::max_element( s->step_ms.begin(), s->step_ms.end() );
    return BORA_OK;
}

}  // extern "C"
