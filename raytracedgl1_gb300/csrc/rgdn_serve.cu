// Serving loop behind rgdn_server_*: continuous batching of frame requests from many camera
// streams onto the batch executor (rgdn_batch.cu).
//
// Threads: callers submit (any thread); a scheduler thread forms steps and enqueues them; a
// completion thread waits for steps in order and stamps their frames done.
//
// Scheduling (the scheduler thread, one step per pass):
//   * a step is started whenever frames are waiting and fewer than stepsInFlight steps are on
//     the GPU, so new frames join the next step while the previous one runs;
//   * candidates are the oldest waiting frame of each stream, in arrival order; a frame whose
//     stream has no memory yet is admitted if the context budget allows (idle streams may be
//     evicted, oldest first), otherwise it waits for memory to free up;
//   * the step takes candidates while it has fewer than maxFramesPerStep frames and its pixels
//     stay within maxPixelsPerStep (the first candidate is always taken);
//   * steps alternate between two CUDA streams; a step waits (cudaStreamWaitEvent) only for an
//     unfinished earlier step on the other CUDA stream that holds one of its camera streams.
// A frame's G-buffer is copied into (or bound to) the stream's planes at the head of its step,
// and PRE_FINAL is copied out after the step when the request asks for it.
#include <algorithm>
#include <limits>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rgdn_host.h"

namespace
{

using Clock = std::chrono::steady_clock;
double now_s() { return std::chrono::duration< double >( Clock::now().time_since_epoch() ).count(); }

enum ReqState : uint32_t
{
    REQ_QUEUED = 100,
    REQ_RUNNING,
    REQ_DONE = RGDN_FRAME_DONE,
    REQ_DROPPED = RGDN_FRAME_DROPPED,
};

struct ServeReq
{
    rgdn_frame_request req;
    uint32_t           state = REQ_QUEUED;
    uint32_t           fi    = 0;
    double             tSubmit = 0, tEnqueue = 0, tDone = 0;
};

struct ServeStream
{
    uint32_t               id = 0, W = 0, H = 0;
    rgdn_stream*           s = nullptr;
    uint32_t               nextFi  = 0;
    std::deque< uint64_t > queue;            // waiting tickets, oldest first
    uint32_t               running = 0;      // frames of this stream in unfinished steps
    int64_t                lastStep = -1;    // step index of its latest scheduled frame
    double                 lastUse  = 0;
    bool                   closing  = false;
};

struct StepRec
{
    int64_t                 index;
    int                     lane;           // which CUDA stream
    cudaEvent_t             done;
    cudaEvent_t             mark[ 4 ] = {}; // timing: start, copies in, kernels, copies out done
    double                  issueMs = 0;    // host time in enqueue_step
    std::vector< uint64_t > tickets;
    std::vector< uint32_t > streams;
    uint64_t                pixels;
};

}  // namespace

struct rgdn_server
{
    rgdn_context*           ctx = nullptr;
    rgdn_server_create_info info{};
    std::mutex              m;
    std::condition_variable cvWork, cvDone;
    std::map< uint32_t, ServeStream >       streams;
    std::unordered_map< uint64_t, ServeReq > reqs;
    std::deque< uint64_t >  arrival;         // waiting tickets in arrival order
    uint32_t                nextStreamId = 1;
    uint64_t                nextTicket   = 1;
    int64_t                 nextStep     = 0;
    std::deque< StepRec >   inflight;
    std::vector< cudaEvent_t > eventPool;
    cudaStream_t            lane[ 2 ] = { nullptr, nullptr };
    std::thread             scheduler, completer;
    bool                    stop = false;
    uint64_t                changes   = 0;      // submissions, completions, closes
    uint64_t                stalledAt = ~0ull;  // `changes` when a pass found nothing to run
    bool                    stalled   = false;  // ... with nothing in flight either
    bool                    forming   = false;  // a step left `arrival` and is not in `inflight` yet
    rgdn_status             error = RGDN_SUCCESS;   // first asynchronous failure
    // statistics
    uint64_t                framesDone = 0, framesDropped = 0, steps = 0, pixelsDone = 0, framesInSteps = 0;
    std::vector< float >    latencies;
    std::vector< float >    issueMs, copyInMs, kernelsMs, copyOutMs;   // per step
    std::vector< cudaEvent_t > timingPool;
    double                  busyStart = -1, busySeconds = 0;
    uint32_t                magic = 0x52475356u;
};

namespace
{

bool valid_server( rgdn_server* s ) { return s && s->magic == 0x52475356u; }

cudaEvent_t take_event( rgdn_server* sv )
{
    if( !sv->eventPool.empty() )
    {
        cudaEvent_t e = sv->eventPool.back();
        sv->eventPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    return cudaEventCreateWithFlags( &e, cudaEventDisableTiming ) == cudaSuccess ? e : nullptr;
}

cudaEvent_t take_timing_event( rgdn_server* sv )
{
    if( !sv->timingPool.empty() )
    {
        cudaEvent_t e = sv->timingPool.back();
        sv->timingPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    return cudaEventCreate( &e ) == cudaSuccess ? e : nullptr;
}

uint64_t stream_bytes( rgdn_server* sv, const ServeStream& st )
{
    rgdn_stream_create_info ci = { st.W, st.H, sv->info.storage };
    uint64_t                b  = 0;
    rgdn_stream_required_bytes( &ci, &b );
    return b;
}

// Admission of a stream without memory (lock held). Evicts idle streams, least recently
// used first, when the budget is short and eviction is enabled.
bool admit( rgdn_server* sv, ServeStream& st )
{
    rgdn_stream_create_info ci = { st.W, st.H, sv->info.storage };
    for( ;; )
    {
        rgdn_status r = rgdn_stream_create( sv->ctx, &ci, &st.s );
        if( r == RGDN_SUCCESS )
        {
            st.nextFi = 0;
            return true;
        }
        st.s = nullptr;
        if( r != RGDN_OUT_OF_BUDGET || !sv->info.evictIdleMs ) return false;
        const double t      = now_s();
        ServeStream* victim = nullptr;
        for( auto& kv : sv->streams )
        {
            ServeStream& o = kv.second;
            if( &o == &st || !o.s || o.running || !o.queue.empty() ) continue;
            if( ( t - o.lastUse ) * 1e3 < (double)sv->info.evictIdleMs ) continue;
            if( !victim || o.lastUse < victim->lastUse ) victim = &o;
        }
        if( !victim ) return false;
        rgdn_stream_destroy( victim->s );
        victim->s = nullptr;
    }
}

// ------------------------------------------------------------------------------------------
// RGDN_HOST_COPY_SM: a frame's pinned host planes copied by one kernel. The planes are split
// into chunks of kChunkBytes, numbered over the planes in order (plane s holds chunks
// first[s] .. first[s + 1] - 1); block b copies chunks b, b + grid, ... with 16-byte loads of
// the device-mapped host pages, four in flight per thread. kGatherBlocks blocks keep about
// 0.5 MB of loads in flight, enough for the host link's rate, and leave the other SMs to the
// kernels of the step on the other lane.
// ------------------------------------------------------------------------------------------
constexpr int      kGatherThreads = 256;
constexpr uint32_t kGatherBlocks  = 32;
constexpr uint64_t kChunkBytes    = 256ull << 10;
struct GatherList
{
    const uint4* src[ RGDN_GBUFFER_PLANES ];
    uint4*       dst[ RGDN_GBUFFER_PLANES ];
    uint64_t     n16[ RGDN_GBUFFER_PLANES ];        // 16-byte units of the plane
    uint32_t     first[ RGDN_GBUFFER_PLANES + 1 ];  // first block of each plane, then the total
    int          count;
};

__global__ void __launch_bounds__( kGatherThreads ) k_gather_host( const GatherList L )
{
    const uint32_t total = L.first[ L.count ];
    int            p     = 0;
    for( uint32_t chunk = blockIdx.x; chunk < total; chunk += gridDim.x )
    {
        while( p + 1 < L.count && L.first[ p + 1 ] <= chunk ) p++;
        const uint64_t per   = kChunkBytes / 16;
        const uint64_t begin = (uint64_t)( chunk - L.first[ p ] ) * per;
        const uint64_t end   = begin + per < L.n16[ p ] ? begin + per : L.n16[ p ];
        const uint4*   src   = L.src[ p ];
        uint4*         dst   = L.dst[ p ];
        uint64_t       i     = begin + threadIdx.x;
        for( ; i + 3 * kGatherThreads < end; i += 4 * kGatherThreads )
        {
            const uint4 a = src[ i ], b = src[ i + kGatherThreads ], c = src[ i + 2 * kGatherThreads ], d = src[ i + 3 * kGatherThreads ];
            dst[ i ]                      = a;
            dst[ i + kGatherThreads ]     = b;
            dst[ i + 2 * kGatherThreads ] = c;
            dst[ i + 3 * kGatherThreads ] = d;
        }
        for( ; i < end; i += kGatherThreads ) dst[ i ] = src[ i ];
    }
}

// The device address of a pinned, device-mapped host buffer (nullptr otherwise)
const void* mapped_host( const void* p )
{
    cudaPointerAttributes at;
    if( cudaPointerGetAttributes( &at, p ) != cudaSuccess )
    {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Adds dst <- src (bytes) to the gather list when the SM loader can take it (device-mapped
// pinned host memory, 16-byte aligned addresses and size); false otherwise
bool gather_add( GatherList& gl, void* dst, const void* src, size_t bytes )
{
    if( gl.count >= RGDN_GBUFFER_PLANES || bytes == 0 || bytes % 16 != 0 || ( (uintptr_t)dst & 15 ) != 0 ) return false;
    const void* m = mapped_host( src );
    if( !m || ( (uintptr_t)m & 15 ) != 0 ) return false;
    const int c       = gl.count++;
    gl.src[ c ]       = static_cast< const uint4* >( m );
    gl.dst[ c ]       = static_cast< uint4* >( dst );
    gl.n16[ c ]       = bytes / 16;
    gl.first[ c + 1 ] = gl.first[ c ] + (uint32_t)( ( bytes + kChunkBytes - 1 ) / kChunkBytes );
    return true;
}

cudaError_t gather_launch( const GatherList& gl, cudaStream_t cs )
{
    if( !gl.count ) return cudaSuccess;
    k_gather_host<<< std::min( gl.first[ gl.count ], kGatherBlocks ), kGatherThreads, 0, cs >>>( gl );
    return cudaGetLastError();
}

void record_done( rgdn_server* sv, ServeReq& r, uint32_t state, double t )
{
    r.state = state;
    r.tDone = t;
    if( state == REQ_DONE )
    {
        sv->framesDone++;
        sv->latencies.push_back( (float)( ( t - r.tSubmit ) * 1e3 ) );
    }
    else sv->framesDropped++;
}

// Enqueues one step (no lock held). Returns the step's completion event.
rgdn_status enqueue_step( rgdn_server* sv, StepRec& rec, std::vector< rgdn_job >& jobs, std::vector< rgdn_stream* >& sts,
                          std::vector< ServeReq* >& rq, std::vector< cudaEvent_t >& waits )
{
    cudaStream_t cs = sv->lane[ rec.lane ];
    for( cudaEvent_t e : waits )
        if( cudaStreamWaitEvent( cs, e, 0 ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    if( rec.mark[ 0 ] && cudaEventRecord( rec.mark[ 0 ], cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    for( size_t k = 0; k < jobs.size(); k++ )
    {
        const rgdn_frame_request& q = rq[ k ]->req;
        GatherList                gl;
        memset( &gl, 0, sizeof( gl ) );
        for( uint32_t fb = 0; fb < RGDN_GBUFFER_PLANES; fb++ )
        {
            if( q.gbufferMode == RGDN_REQUEST_BIND )
            {
                // NULL restores the stream's own plane
                rgdn_status r = rgdn_stream_bind_framebuffer( sts[ k ], fb, jobs[ k ].frameIndex, const_cast< void* >( q.gbuffer[ fb ] ) );
                if( r != RGDN_SUCCESS ) return r;
                continue;
            }
            if( !q.gbuffer[ fb ] ) continue;
            rgdn_image img;
            rgdn_status r = rgdn_stream_get_framebuffer( sts[ k ], fb, jobs[ k ].frameIndex, &img );
            if( r != RGDN_SUCCESS ) return r;
            const size_t bytes = (size_t)img.pitch_bytes * img.height;
            if( sv->info.hostCopy == RGDN_HOST_COPY_SM && gather_add( gl, img.data, q.gbuffer[ fb ], bytes ) ) continue;
            if( cudaMemcpyAsync( img.data, q.gbuffer[ fb ], bytes, cudaMemcpyDefault, cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
        }
        if( gl.count )
        {
            if( gather_launch( gl, cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
            sv->ctx->launches.fetch_add( 1, std::memory_order_relaxed );
        }
    }
    if( rec.mark[ 1 ] && cudaEventRecord( rec.mark[ 1 ], cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    rgdn_status r = rgdn_submit_batch( sv->ctx, jobs.data(), (uint32_t)jobs.size(), (rgdn_cuda_stream)cs );
    if( r != RGDN_SUCCESS ) return r;
    if( rec.mark[ 2 ] && cudaEventRecord( rec.mark[ 2 ], cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    for( size_t k = 0; k < jobs.size(); k++ )
    {
        if( !rq[ k ]->req.preFinalOut ) continue;
        rgdn_image img;
        if( ( r = rgdn_stream_get_framebuffer( sts[ k ], RGDN_FB_PRE_FINAL, jobs[ k ].frameIndex, &img ) ) != RGDN_SUCCESS ) return r;
        if( cudaMemcpyAsync( rq[ k ]->req.preFinalOut, img.data, (size_t)img.pitch_bytes * img.height, cudaMemcpyDefault, cs ) != cudaSuccess )
            return RGDN_DEVICE_ERROR;
    }
    if( rec.mark[ 3 ] && cudaEventRecord( rec.mark[ 3 ], cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    return cudaEventRecord( rec.done, cs ) == cudaSuccess ? RGDN_SUCCESS : RGDN_DEVICE_ERROR;
}

void scheduler_loop( rgdn_server* sv )
{
    cudaSetDevice( sv->ctx->device );
    const uint32_t maxFrames = sv->info.maxFramesPerStep ? std::min( sv->info.maxFramesPerStep, (uint32_t)rgdn::MAX_BATCH ) : (uint32_t)rgdn::MAX_BATCH;
    const uint32_t inFlight  = sv->info.stepsInFlight ? std::min( sv->info.stepsInFlight, 3u ) : 2u;
    std::unique_lock< std::mutex > lk( sv->m );
    for( ;; )
    {
        sv->cvWork.wait( lk, [ & ] {
            return sv->stop || ( !sv->arrival.empty() && sv->inflight.size() < inFlight && sv->changes != sv->stalledAt );
        } );
        if( sv->stop )
        {
            // frames that could never be admitted: dropped
            const double t = now_s();
            for( uint64_t tk : sv->arrival )
            {
                ServeReq& q = sv->reqs[ tk ];
                sv->streams[ q.req.stream ].queue.clear();
                record_done( sv, q, REQ_DROPPED, t );
            }
            sv->arrival.clear();
            sv->cvDone.notify_all();
            break;
        }

        // form the step
        StepRec rec;
        rec.index  = sv->nextStep;
        rec.lane   = (int)( rec.index & 1 );
        rec.pixels = 0;
        std::vector< rgdn_job >     jobs;
        std::vector< rgdn_stream* > sts;
        std::vector< ServeReq* >    rq;
        std::vector< cudaEvent_t >  waits;
        std::vector< uint64_t >     keep;
        bool                        full = false;
        for( uint64_t t : sv->arrival )
        {
            ServeReq&    r  = sv->reqs[ t ];
            ServeStream& st = sv->streams[ r.req.stream ];
            const bool   oldest = st.queue.front() == t;
            bool         take   = !full && oldest && st.lastStep != rec.index;
            if( take && !st.s && !admit( sv, st ) ) take = false;
            const uint64_t px = (uint64_t)st.W * st.H;
            if( take && !jobs.empty() &&
                ( jobs.size() >= maxFrames || ( sv->info.maxPixelsPerStep && rec.pixels + px > sv->info.maxPixelsPerStep ) ) )
            {
                take = false;
                full = true;
            }
            if( !take )
            {
                keep.push_back( t );
                continue;
            }
            // a step on the other lane still holding this stream must finish first
            for( const StepRec& o : sv->inflight )
                if( o.lane != rec.lane && o.index == st.lastStep &&
                    std::find( waits.begin(), waits.end(), o.done ) == waits.end() )
                    waits.push_back( o.done );
            r.state    = REQ_RUNNING;
            r.fi       = st.nextFi;
            r.tEnqueue = now_s();
            st.nextFi ^= 1u;
            st.queue.pop_front();
            st.running++;
            st.lastStep = rec.index;
            st.lastUse  = r.tEnqueue;
            jobs.push_back( { st.s, r.fi, &r.req.params } );
            sts.push_back( st.s );
            rq.push_back( &r );
            rec.tickets.push_back( t );
            rec.streams.push_back( st.id );
            rec.pixels += px;
        }
        if( jobs.empty() )
        {
            // nothing admissible now: wait for a change (a completion frees memory, a stream
            // closes, a frame arrives)
            sv->stalledAt = sv->changes;
            sv->stalled   = sv->inflight.empty();
            sv->cvDone.notify_all();
            continue;
        }
        sv->stalled = false;
        sv->arrival.assign( keep.begin(), keep.end() );
        rec.done = take_event( sv );
        for( cudaEvent_t& e : rec.mark ) e = take_timing_event( sv );
        sv->nextStep++;
        // its frames are in neither `arrival` nor `inflight` while the lock is released
        sv->forming = true;
        lk.unlock();
        const double tIssue = now_s();
        rgdn_status  r      = rec.done ? enqueue_step( sv, rec, jobs, sts, rq, waits ) : RGDN_DEVICE_ERROR;
        rec.issueMs         = ( now_s() - tIssue ) * 1e3;
        lk.lock();
        sv->forming = false;
        if( r != RGDN_SUCCESS )
        {
            // the frames cannot complete: report them dropped and remember the failure
            if( sv->error == RGDN_SUCCESS ) sv->error = r;
            const double t = now_s();
            for( size_t k = 0; k < rec.tickets.size(); k++ )
            {
                ServeReq& q = sv->reqs[ rec.tickets[ k ] ];
                record_done( sv, q, REQ_DROPPED, t );
                sv->streams[ rec.streams[ k ] ].running--;
            }
            if( rec.done ) sv->eventPool.push_back( rec.done );
            for( cudaEvent_t e : rec.mark )
                if( e ) sv->timingPool.push_back( e );
            sv->cvDone.notify_all();
            continue;
        }
        if( sv->inflight.empty() ) sv->busyStart = now_s();
        sv->inflight.push_back( std::move( rec ) );
        sv->cvDone.notify_all();   // wakes the completion thread
    }
}

void completion_loop( rgdn_server* sv )
{
    cudaSetDevice( sv->ctx->device );
    std::unique_lock< std::mutex > lk( sv->m );
    for( ;; )
    {
        sv->cvDone.wait( lk, [ & ] { return sv->stop || !sv->inflight.empty(); } );
        if( sv->inflight.empty() )
        {
            if( sv->stop ) break;
            continue;
        }
        cudaEvent_t e = sv->inflight.front().done;
        lk.unlock();
        const cudaError_t ce = cudaEventSynchronize( e );
        const double      t  = now_s();
        lk.lock();
        StepRec rec = std::move( sv->inflight.front() );
        sv->inflight.pop_front();
        if( ce != cudaSuccess && sv->error == RGDN_SUCCESS ) sv->error = RGDN_DEVICE_ERROR;
        for( size_t k = 0; k < rec.tickets.size(); k++ )
        {
            ServeReq& q = sv->reqs[ rec.tickets[ k ] ];
            record_done( sv, q, ce == cudaSuccess ? REQ_DONE : REQ_DROPPED, t );
            ServeStream& st = sv->streams[ rec.streams[ k ] ];
            st.running--;
        }
        if( ce == cudaSuccess && rec.mark[ 0 ] && rec.mark[ 1 ] && rec.mark[ 2 ] && rec.mark[ 3 ] )
        {
            float a = 0, b = 0, c = 0;
            if( cudaEventElapsedTime( &a, rec.mark[ 0 ], rec.mark[ 1 ] ) == cudaSuccess &&
                cudaEventElapsedTime( &b, rec.mark[ 1 ], rec.mark[ 2 ] ) == cudaSuccess &&
                cudaEventElapsedTime( &c, rec.mark[ 2 ], rec.mark[ 3 ] ) == cudaSuccess )
            {
                sv->copyInMs.push_back( a );
                sv->kernelsMs.push_back( b );
                sv->copyOutMs.push_back( c );
            }
        }
        sv->issueMs.push_back( (float)rec.issueMs );
        for( cudaEvent_t e : rec.mark )
            if( e ) sv->timingPool.push_back( e );
        sv->steps++;
        sv->framesInSteps += rec.tickets.size();
        sv->pixelsDone += rec.pixels;
        if( sv->inflight.empty() && sv->busyStart >= 0 )
        {
            sv->busySeconds += t - sv->busyStart;
            sv->busyStart = -1;
        }
        sv->eventPool.push_back( rec.done );
        sv->changes++;
        sv->cvDone.notify_all();
        sv->cvWork.notify_all();
    }
}

float percentile( std::vector< float > v, double q )
{
    if( v.empty() ) return 0.0f;
    std::sort( v.begin(), v.end() );
    const size_t i = (size_t)( q * (double)( v.size() - 1 ) + 0.5 );
    return v[ std::min( i, v.size() - 1 ) ];
}

// The q-quantile over every finished request, each dropped one counted as an unbounded latency:
// +infinity once the dropped requests reach past the quantile.
float percentile_all( std::vector< float > v, uint64_t dropped, double q )
{
    const uint64_t n = (uint64_t)v.size() + dropped;
    if( n == 0 ) return 0.0f;
    std::sort( v.begin(), v.end() );
    const uint64_t i = std::min< uint64_t >( (uint64_t)( q * (double)( n - 1 ) + 0.5 ), n - 1 );
    return i < v.size() ? v[ i ] : std::numeric_limits< float >::infinity();
}

}  // namespace

extern "C" {

rgdn_status rgdn_server_create( rgdn_context* ctx, const rgdn_server_create_info* info, rgdn_server** out )
{
    if( !rgdn::valid_ctx( ctx ) ) return RGDN_WRONG_INSTANCE;
    if( !info || !out || info->storage > RGDN_STORAGE_BF16 || info->maxFramesPerStep > (uint32_t)rgdn::MAX_BATCH || info->stepsInFlight > 3 ||
        info->hostCopy > RGDN_HOST_COPY_SM )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    cudaSetDevice( ctx->device );
    rgdn_server* sv = new( std::nothrow ) rgdn_server();
    if( !sv ) return RGDN_INTERNAL_ERROR;
    sv->ctx  = ctx;
    sv->info = *info;
    for( int i = 0; i < 2; i++ )
        if( cudaStreamCreateWithFlags( &sv->lane[ i ], cudaStreamNonBlocking ) != cudaSuccess )
        {
            for( int k = 0; k < i; k++ ) cudaStreamDestroy( sv->lane[ k ] );
            delete sv;
            return RGDN_DEVICE_ERROR;
        }
    sv->scheduler = std::thread( scheduler_loop, sv );
    sv->completer = std::thread( completion_loop, sv );
    *out          = sv;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_drain( rgdn_server* sv )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    std::unique_lock< std::mutex > lk( sv->m );
    sv->cvDone.wait( lk, [ & ] {
        return !sv->forming && sv->inflight.empty() && ( sv->arrival.empty() || ( sv->stalled && sv->stalledAt == sv->changes ) );
    } );
    if( sv->error != RGDN_SUCCESS ) return sv->error;
    // frames left waiting can run only after memory frees up (rgdn_server_close_stream)
    return sv->arrival.empty() ? RGDN_SUCCESS : RGDN_OUT_OF_BUDGET;
}

rgdn_status rgdn_server_destroy( rgdn_server* sv )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    rgdn_server_drain( sv );
    {
        std::lock_guard< std::mutex > g( sv->m );
        sv->stop = true;
    }
    sv->cvWork.notify_all();
    sv->cvDone.notify_all();
    sv->scheduler.join();
    sv->completer.join();
    cudaSetDevice( sv->ctx->device );
    for( auto& kv : sv->streams )
        if( kv.second.s ) rgdn_stream_destroy( kv.second.s );
    for( cudaEvent_t e : sv->eventPool ) cudaEventDestroy( e );
    for( cudaEvent_t e : sv->timingPool ) cudaEventDestroy( e );
    for( int i = 0; i < 2; i++ ) cudaStreamDestroy( sv->lane[ i ] );
    sv->magic = 0;
    delete sv;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_open_stream( rgdn_server* sv, uint32_t width, uint32_t height, uint32_t* outId )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    if( !outId || width < 2 || height < 1 || ( width & 1 ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    std::lock_guard< std::mutex > g( sv->m );
    ServeStream st;
    st.id = sv->nextStreamId++;
    st.W  = width;
    st.H  = height;
    sv->streams[ st.id ] = st;
    *outId               = st.id;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_close_stream( rgdn_server* sv, uint32_t id )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    std::unique_lock< std::mutex > lk( sv->m );
    auto it = sv->streams.find( id );
    if( it == sv->streams.end() || it->second.closing ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    it->second.closing = true;
    sv->cvDone.wait( lk, [ & ] { return it->second.queue.empty() && it->second.running == 0; } );
    if( it->second.s )
    {
        cudaSetDevice( sv->ctx->device );
        rgdn_stream_destroy( it->second.s );
    }
    sv->streams.erase( it );
    sv->changes++;
    sv->cvWork.notify_all();   // memory freed: waiting admissions may proceed
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_submit( rgdn_server* sv, const rgdn_frame_request* req, uint64_t* outTicket )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    if( !req || !outTicket || req->gbufferMode > RGDN_REQUEST_BIND ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    rgdn_status r = rgdn::check_params( &req->params );
    if( r != RGDN_SUCCESS ) return r;
    if( req->params.flags & ( RGDN_FLAG_PLAIN | RGDN_FLAG_EXACT_MATH | RGDN_FLAG_TMA_STAGING ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    std::lock_guard< std::mutex > g( sv->m );
    auto it = sv->streams.find( req->stream );
    if( it == sv->streams.end() || it->second.closing ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    ServeStream& st = it->second;
    const double t  = now_s();
    // latest frames win: drop the oldest waiting frames beyond the stream's allowance
    while( sv->info.maxQueuedPerStream && st.queue.size() >= sv->info.maxQueuedPerStream )
    {
        const uint64_t old = st.queue.front();
        st.queue.pop_front();
        sv->arrival.erase( std::find( sv->arrival.begin(), sv->arrival.end(), old ) );
        record_done( sv, sv->reqs[ old ], REQ_DROPPED, t );
    }
    const uint64_t ticket = sv->nextTicket++;
    ServeReq&      q      = sv->reqs[ ticket ];
    q.req                 = *req;
    q.tSubmit             = t;
    st.queue.push_back( ticket );
    sv->arrival.push_back( ticket );
    *outTicket = ticket;
    sv->changes++;
    sv->cvWork.notify_one();
    sv->cvDone.notify_all();
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_wait( rgdn_server* sv, uint64_t ticket, uint32_t timeoutMs, rgdn_frame_result* out )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    if( !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    std::unique_lock< std::mutex > lk( sv->m );
    if( sv->reqs.find( ticket ) == sv->reqs.end() ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    // the ticket is looked up again after every wake-up: a submit on another thread may rehash
    // the map while the lock is released (invalidating iterators), and another waiter on the
    // same ticket may already have taken and erased it
    auto finished = [ & ] {
        const auto f = sv->reqs.find( ticket );
        return f == sv->reqs.end() || f->second.state == REQ_DONE || f->second.state == REQ_DROPPED;
    };
    if( !sv->cvDone.wait_for( lk, std::chrono::milliseconds( timeoutMs ), finished ) ) return RGDN_TIMEOUT;
    const auto it = sv->reqs.find( ticket );
    if( it == sv->reqs.end() ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    const ServeReq& q = it->second;
    out->state        = q.state;
    out->frameIndex   = q.fi;
    out->latencyMs    = (float)( ( q.tDone - q.tSubmit ) * 1e3 );
    out->queueMs      = q.tEnqueue > 0 ? (float)( ( q.tEnqueue - q.tSubmit ) * 1e3 ) : out->latencyMs;
    sv->reqs.erase( it );
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_stats_get( rgdn_server* sv, rgdn_server_stats* out )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    if( !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    std::lock_guard< std::mutex > g( sv->m );
    memset( out, 0, sizeof( *out ) );
    out->framesDone    = sv->framesDone;
    out->framesDropped = sv->framesDropped;
    out->steps         = sv->steps;
    out->pixelsDone    = sv->pixelsDone;
    out->queuedFrames  = (uint32_t)sv->arrival.size();
    for( auto& kv : sv->streams )
        if( kv.second.s )
        {
            out->residentStreams++;
            out->residentBytes += stream_bytes( sv, kv.second );
        }
    out->p50Ms             = percentile( sv->latencies, 0.50 );
    out->p99Ms             = percentile( sv->latencies, 0.99 );
    out->maxMs             = percentile( sv->latencies, 1.0 );
    out->p99AllMs          = percentile_all( sv->latencies, sv->framesDropped, 0.99 );
    out->dropRate          = ( sv->framesDone + sv->framesDropped )
                                 ? (float)( (double)sv->framesDropped / (double)( sv->framesDone + sv->framesDropped ) )
                                 : 0.0f;
    out->meanFramesPerStep = sv->steps ? (float)sv->framesInSteps / (float)sv->steps : 0.0f;
    out->busySeconds       = sv->busySeconds + ( sv->busyStart >= 0 ? now_s() - sv->busyStart : 0.0 );
    out->issueP50Ms        = percentile( sv->issueMs, 0.50 );
    out->issueP99Ms        = percentile( sv->issueMs, 0.99 );
    out->copyInP50Ms       = percentile( sv->copyInMs, 0.50 );
    out->copyInP99Ms       = percentile( sv->copyInMs, 0.99 );
    out->kernelsP50Ms      = percentile( sv->kernelsMs, 0.50 );
    out->kernelsP99Ms      = percentile( sv->kernelsMs, 0.99 );
    out->copyOutP50Ms      = percentile( sv->copyOutMs, 0.50 );
    out->copyOutP99Ms      = percentile( sv->copyOutMs, 0.99 );
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_stats_reset( rgdn_server* sv )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    std::lock_guard< std::mutex > g( sv->m );
    sv->framesDone = sv->framesDropped = sv->steps = sv->pixelsDone = sv->framesInSteps = 0;
    sv->latencies.clear();
    sv->issueMs.clear();
    sv->copyInMs.clear();
    sv->kernelsMs.clear();
    sv->copyOutMs.clear();
    sv->busySeconds = 0;
    if( sv->busyStart >= 0 ) sv->busyStart = now_s();
    return RGDN_SUCCESS;
}

rgdn_status rgdn_server_get_stream( rgdn_server* sv, uint32_t id, rgdn_stream** out )
{
    if( !valid_server( sv ) ) return RGDN_WRONG_INSTANCE;
    if( !out ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    std::lock_guard< std::mutex > g( sv->m );
    auto it = sv->streams.find( id );
    if( it == sv->streams.end() ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    *out = it->second.s;
    return RGDN_SUCCESS;
}

rgdn_status rgdn_copy_host_planes( void* const* dst, const void* const* src, const size_t* bytes, uint32_t count, uint32_t hostCopy,
                                   rgdn_cuda_stream cudaStream )
{
    if( !dst || !src || !bytes || count == 0 || count > RGDN_GBUFFER_PLANES ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    if( hostCopy != RGDN_HOST_COPY_ENGINE && hostCopy != RGDN_HOST_COPY_SM ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    for( uint32_t k = 0; k < count; k++ )
        if( !dst[ k ] || !src[ k ] ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    const cudaStream_t cs = (cudaStream_t)cudaStream;
    GatherList         gl;
    memset( &gl, 0, sizeof( gl ) );
    for( uint32_t k = 0; k < count; k++ )
    {
        if( hostCopy == RGDN_HOST_COPY_SM && gather_add( gl, dst[ k ], src[ k ], bytes[ k ] ) ) continue;
        if( bytes[ k ] && cudaMemcpyAsync( dst[ k ], src[ k ], bytes[ k ], cudaMemcpyDefault, cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
    }
    return gather_launch( gl, cs ) == cudaSuccess ? RGDN_SUCCESS : RGDN_DEVICE_ERROR;
}

}  // extern "C"
