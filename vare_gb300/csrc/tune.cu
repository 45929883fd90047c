// Launch-shape autotuner.
//
// Some kernels have several launch shapes that compute bit-identical results - the multigrid
// passes that reduce nothing (level 0's warps per block, levels 1 and 2's threads per block) -
// and whose best shape depends on the device and the amount of work. For each (kernel group,
// device, size class = floor(log2 units)) the tuner times every candidate shape on live
// launches (CUDA events on the launching stream, kSamples launches each, candidates in turn),
// then keeps the one with the smallest median for every later launch of that class. Because
// every candidate computes the same bits, tuning changes no result: a simulation gives the
// same bits with tuning on or off, alone or in a batch. Kernels whose shape fixes the
// summation order of a reduction are never tuned.
//
// The table can be loaded from and saved to a text file (BORA_TUNE_FILE: one line per entry,
// "group device size_class variant median_ms"), so a deployment reuses measured shapes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/bora_flip.h"
#include "bora_internal.h"

namespace {

constexpr int kSamples = 3;

struct Entry
{
    int nvar = 0;
    int chosen = -1;
    std::vector<std::vector<float>> ms;  // samples per variant
    std::vector<int> inflight;           // timed launches not yet resolved, per variant
    double best_ms = 0.0;
};

struct Pending
{
    int group, units, variant, device;
    cudaEvent_t a, b;
};

struct Tuner
{
    std::mutex mu;
    int mode = 1;  // 1: tune, 0: the default shape everywhere
    bool loaded = false;
    std::map<std::tuple<int, int, int>, Entry> table;  // (group, device, size class)
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;

    static int size_class( int units ) { int c = 0; for( int u = std::max( units, 1 ); u > 1; u >>= 1 ) ++c; return c; }

    void load_locked()
    {
        if( loaded ) return;
        loaded = true;
        const char* path = std::getenv( "BORA_TUNE_FILE" );
        if( !path || !*path ) return;
        FILE* f = std::fopen( path, "r" );
        if( !f ) return;
        int g, d, c, v;
        double m;
        while( std::fscanf( f, "%d %d %d %d %lf", &g, &d, &c, &v, &m ) == 5 )
        {
            if( g < 0 || g >= kBoraTuneGroups || v < 0 || v >= bora_tune_variants( g ) ) continue;
            Entry& e = table[std::make_tuple( g, d, c )];
            e.nvar = bora_tune_variants( g );
            e.chosen = v;
            e.best_ms = m;
        }
        std::fclose( f );
    }

    void save_locked()
    {
        const char* path = std::getenv( "BORA_TUNE_FILE" );
        if( !path || !*path ) return;
        FILE* f = std::fopen( path, "w" );
        if( !f ) return;
        for( const auto& kv : table )
            if( kv.second.chosen >= 0 )
                std::fprintf( f, "%d %d %d %d %.6f\n", std::get<0>( kv.first ), std::get<1>( kv.first ),
                              std::get<2>( kv.first ), kv.second.chosen, kv.second.best_ms );
        std::fclose( f );
    }

    Entry& entry_locked( int group, int device, int units )
    {
        load_locked();
        Entry& e = table[std::make_tuple( group, device, size_class( units ) )];
        if( e.nvar == 0 ) e.nvar = bora_tune_variants( group );
        if( (int)e.ms.size() != e.nvar ) e.ms.assign( e.nvar, {} );
        if( (int)e.inflight.size() != e.nvar ) e.inflight.assign( e.nvar, 0 );
        return e;
    }

    cudaEvent_t take()
    {
        if( !pool.empty() ) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e = nullptr;
        if( cudaEventCreate( &e ) != cudaSuccess ) { cudaGetLastError(); return nullptr; }
        return e;
    }
};

Tuner& tuner()
{
    static Tuner* t = new Tuner;  // never destroyed: launches may still consult it at exit
    return *t;
}

int current_device()
{
    int d = 0;
    cudaGetDevice( &d );
    return d;
}

}  // namespace

int bora_tune_variants( int group )
{
    switch( group )
    {
    case kBoraTuneL0: case kBoraTuneL0Batch: return 3;  // 2, 4, 8 warps (tiles) per block
    case kBoraTuneL1: case kBoraTuneL2: case kBoraTuneL1Batch: case kBoraTuneL2Batch: return 4;  // 64 .. 512 threads
    default: return 1;
    }
}

int bora_tune_default( int group )
{
    switch( group )
    {
    case kBoraTuneL0: case kBoraTuneL0Batch: return 1;
    case kBoraTuneL1: case kBoraTuneL2: case kBoraTuneL1Batch: case kBoraTuneL2Batch: return 2;
    default: return 0;
    }
}

BoraTunePick bora_tune_pick( int group, int units )
{
    BoraTunePick p{ bora_tune_default( group ), false };
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk( t.mu );
    if( !t.mode ) return p;
    Entry& e = t.entry_locked( group, current_device(), units );
    if( e.chosen >= 0 ) { p.variant = e.chosen; return p; }
    // the candidate with the fewest samples so far, counting launches still in flight
    int v = 0;
    for( int q = 1; q < e.nvar; ++q )
        if( e.ms[q].size() + e.inflight[q] < e.ms[v].size() + e.inflight[v] ) v = q;
    p.variant = v;
    p.timed = true;
    return p;
}

BoraTuneTimer::BoraTuneTimer( const BoraTunePick& p, int group, int units, cudaStream_t st )
    : timed( p.timed ), group( group ), units( units ), variant( p.variant ), st( st )
{
    if( !timed ) return;
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk( t.mu );
    a = t.take();
    if( a ) cudaEventRecord( a, st );
}

BoraTuneTimer::~BoraTuneTimer()
{
    if( !timed || !a ) return;
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk( t.mu );
    cudaEvent_t b = t.take();
    if( !b ) { t.pool.push_back( a ); return; }
    cudaEventRecord( b, st );
    const int dev = current_device();
    t.pending.push_back( Pending{ group, units, variant, dev, a, b } );
    Entry& e = t.entry_locked( group, dev, units );
    if( variant < e.nvar ) ++e.inflight[variant];
}

void bora_tune_resolve()
{
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk( t.mu );
    std::vector<Pending> keep;
    bool frozen = false;
    for( const Pending& p : t.pending )
    {
        const cudaError_t q = cudaEventQuery( p.b );
        if( q == cudaErrorNotReady ) { keep.push_back( p ); continue; }
        float ms = 0.f;
        const bool ok = q == cudaSuccess && cudaEventElapsedTime( &ms, p.a, p.b ) == cudaSuccess;
        cudaGetLastError();
        t.pool.push_back( p.a );
        t.pool.push_back( p.b );
        if( !ok ) continue;
        Entry& e = t.entry_locked( p.group, p.device, p.units );
        if( p.variant < e.nvar && e.inflight[p.variant] > 0 ) --e.inflight[p.variant];
        if( e.chosen >= 0 || p.variant >= e.nvar ) continue;
        e.ms[p.variant].push_back( ms );
        bool done = true;
        for( const auto& v : e.ms ) done = done && v.size() >= (size_t)kSamples;
        if( !done ) continue;
        int best = 0;
        double best_ms = 0.0;
        for( int v = 0; v < e.nvar; ++v )
        {
            std::vector<float> s = e.ms[v];
            std::sort( s.begin(), s.end() );
            const double med = s[s.size() / 2];
            if( v == 0 || med < best_ms ) { best = v; best_ms = med; }
        }
        e.chosen = best;
        e.best_ms = best_ms;
        frozen = true;
    }
    t.pending.swap( keep );
    if( frozen ) t.save_locked();
}

extern "C" {

int bora_flip_set_tuning( int mode )
{
    if( mode != 0 && mode != 1 ) return BORA_ERR_INVALID_ARG;
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk( t.mu );
    t.mode = mode;
    return BORA_OK;
}

int bora_flip_tune_table( char* buf, size_t cap, size_t* len )
{
    if( !len || ( cap > 0 && !buf ) ) return BORA_ERR_INVALID_ARG;
    Tuner& t = tuner();
    std::string out;
    {
        std::lock_guard<std::mutex> lk( t.mu );
        t.load_locked();
        char line[160];
        for( const auto& kv : t.table )
        {
            const Entry& e = kv.second;
            std::snprintf( line, sizeof( line ), "%d %d %d %d %.6f\n", std::get<0>( kv.first ), std::get<1>( kv.first ),
                           std::get<2>( kv.first ), e.chosen, e.best_ms );
            out += line;
        }
    }
    *len = out.size();
    if( out.size() + 1 > cap ) return cap == 0 ? BORA_OK : BORA_ERR_CAPACITY;
    std::memcpy( buf, out.c_str(), out.size() + 1 );
    return BORA_OK;
}

}  // extern "C"
