// Batch executor behind rgdn_submit_batch: many streams' frames of uneven size advance one
// frame each in one step, with one persistent launch per stage.
//
// The reference denoises one camera stream per call (Denoiser::Denoise, Source/Denoiser.cpp:
// 64-255, then Tonemapping::CalculateExposure, Source/Tonemapping.cpp:59-165); a step here runs
// the same stages in the same order for up to MAX_BATCH frames:
//
//   H2D copy of the step table (BatchConst) into the constant slot of the two kernel modules
//   gradient samples, gradient a-trous 0..3        (frames with gradients)
//   temporal accumulation, anti-firefly, variance  (every frame)
//   a-trous 0 .. max(niter)-1                      (frames with niter > i; a frame's last
//                                                   iteration composes and bins its histogram)
//   luminance average                              (every frame)
//
// Every launch has a fixed grid (resident blocks per SM x SMs) and reads its tile table from
// the slot, so the captured graph of a step is valid for any set of frames with the same launch
// sequence; a step then costs the two table copies and one graph launch.
//
// Slots: each kernel module has BATCH_SLOTS constant slots. They and their pinned host tables
// are a per-device resource shared by every context of the process; steps take them in turn,
// and a step waits on the host until the slot's previous step has finished.
//
// Groups: the step's frames run in groups of consecutive frames of at most groupPixels pixels,
// each group through every stage before the next group starts. A frame of at least
// singlePixels pixels is a group of its own and runs on the single-frame kernels, whose frame
// arguments are kernel parameters: read from the constant
// table with a job index known only at run time, the same fields cost the batched kernels
// registers (the batched a-trous and variance builds spill 2-7 times the bytes of the
// single-frame ones) and their large frames ran 5-13 % slower per pixel. A step with such a
// group is launched directly rather than replayed from a graph, since that group's parameters
// change every step; at a frame of a million pixels or more the launches stay ahead of the GPU.
// One-frame groups take turns on the caller's stream and kSideLanes more (enqueue_step).
//
// Autotuning: the first 15 steps of a storage mode time every candidate tile shape (and, for
// the a-trous kernel, the register budget and the fusion depth) per launch on the frames being
// submitted; the fastest candidate per launch is kept. The next 8 steps time whole steps at each
// candidate grouping (kGroupCand) and keep the fastest. Candidates compute identical values per
// pixel, so tuning changes no result. Then steps switch to graph replay.
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <vector>

#include "rgdn_host.h"

namespace rgdn
{
namespace
{

// tuning steps: kTuneRounds passes over the candidates; the first pass only warms up (module
// loading, clocks) and is not scored
constexpr int kTuneRounds = 3;
// RGDN_TILE_*: 32x8, 16x16 and 64x4 tiles of 256 threads; 32x4 tiles of 128 threads, whose
// kernels are built for 7 resident blocks per SM
const dim3    kShapes[ 5 ] = { dim3( 32, 8 ), dim3( 16, 16 ), dim3( 64, 4 ), dim3( 32, 4 ), dim3( 32, 8 ) };

size_t table_bytes( int n ) { return offsetof( BatchConst, jobs ) + sizeof( FrameArgs ) * (size_t)n; }

// the launch sequence of one group of a step's frames (jobs [j0, j1) of the table)
struct GroupKey
{
    int j0, j1, single, anyGrad, maxIter, gpm;   // single: one frame, on the single-frame kernels
    int hm[ MAX_ATROUS_ITERATIONS ];
    int tiles[ BS_COUNT ];   // the grid of one-tile-per-block launches (occ 7, pair), else 0
};
// the launch sequence of a step: what a captured graph depends on (zero-filled before it is
// set, so that memcmp compares it)
struct GraphKey
{
    int      storage, ng;
    int      shape[ BS_COUNT ];
    int      occ[ BS_COUNT ];
    GroupKey g[ MAX_BATCH ];
};
bool same_key( const GraphKey& a, const GraphKey& b ) { return memcmp( &a, &b, sizeof( GraphKey ) ) == 0; }

// per-device constant slots and their pinned host tables
struct DeviceSlots
{
    std::mutex  m;
    bool        ready = false;
    int         next  = 0;
    BatchConst* host[ BATCH_SLOTS ] = {};
    cudaEvent_t done[ BATCH_SLOTS ] = {};
    bool        used[ BATCH_SLOTS ] = {};
    void*       mode[ 4 ][ BATCH_SLOTS ] = {};   // c_batch slot of each storage's mode module
    void*       fast[ 4 ][ BATCH_SLOTS ] = {};   // ... and of its FAST module
};
constexpr int kMaxDevices = 64;
DeviceSlots   g_slots[ kMaxDevices ];

typedef cudaError_t ( *BatchLauncher )( int, int, int, dim3, int, cudaStream_t );
typedef int ( *BpsFn )( int );
typedef void* ( *SlotFn )( int );

BatchLauncher batch_launcher( uint32_t storage, int stage )
{
    const bool fast = is_batch_fast_stage( stage );
    switch( storage )
    {
        case RGDN_STORAGE_REF: return fast ? launch_batch_fast_ref : launch_batch_ref;
        case RGDN_STORAGE_FP32: return fast ? launch_batch_fast_f32 : launch_batch_f32;
        case RGDN_STORAGE_FP16: return fast ? launch_batch_fast_f16 : launch_batch_f16;
        case RGDN_STORAGE_BF16: return fast ? launch_batch_fast_bf16 : launch_batch_bf16;
        default: return nullptr;
    }
}
BpsFn bps_fn( uint32_t storage, int stage )
{
    const bool fast = is_batch_fast_stage( stage & 0xff );
    switch( storage )
    {
        case RGDN_STORAGE_REF: return fast ? batch_blocks_per_sm_fast_ref : batch_blocks_per_sm_ref;
        case RGDN_STORAGE_FP32: return fast ? batch_blocks_per_sm_fast_f32 : batch_blocks_per_sm_f32;
        case RGDN_STORAGE_FP16: return fast ? batch_blocks_per_sm_fast_f16 : batch_blocks_per_sm_f16;
        case RGDN_STORAGE_BF16: return fast ? batch_blocks_per_sm_fast_bf16 : batch_blocks_per_sm_bf16;
        default: return nullptr;
    }
}

// slot set-up on the current device (lock held)
bool slots_ready( DeviceSlots& ds )
{
    if( ds.ready ) return true;
    const SlotFn modeFn[ 4 ] = { batch_slot_ref, batch_slot_f32, batch_slot_f16, batch_slot_bf16 };
    const SlotFn fastFn[ 4 ] = { batch_slot_fast_ref, batch_slot_fast_f32, batch_slot_fast_f16, batch_slot_fast_bf16 };
    for( int s = 0; s < BATCH_SLOTS; s++ )
    {
        if( !ds.host[ s ] )
        {
            void* p = nullptr;
            if( cudaMallocHost( &p, sizeof( BatchConst ) ) != cudaSuccess ) return false;
            memset( p, 0, sizeof( BatchConst ) );
            ds.host[ s ] = static_cast< BatchConst* >( p );
        }
        if( !ds.done[ s ] && cudaEventCreateWithFlags( &ds.done[ s ], cudaEventDisableTiming ) != cudaSuccess ) return false;
        for( int m = 0; m < 4; m++ )
        {
            ds.mode[ m ][ s ] = modeFn[ m ]( s );
            ds.fast[ m ][ s ] = fastFn[ m ]( s );
            if( !ds.mode[ m ][ s ] || !ds.fast[ m ][ s ] ) return false;
        }
    }
    ds.ready = true;
    return true;
}

struct Config
{
    int      shape[ BS_COUNT ];   // index into kShapes (BS_GRADIENT stays 32x8)
    int      occ[ BS_COUNT ];     // a-trous kinds: resident blocks per SM the kernel is built for (3, 4)
    bool     graphs;
    uint64_t groupPixels;         // 0 = no bound on a group's pixels
    uint64_t singlePixels;        // frames of at least this many pixels run alone (0 = never)
};

// kind -2: a whole step (the group-size phase)
struct Probe
{
    int         kind, cand;
    double      pixels;
    cudaEvent_t a, b;
    bool        scored;
};

// Groupings the second tuning phase times, as whole steps (group pixels, single-frame pixels):
// the whole step as one group; groups of about one 2560x1440 frame; frames of 1280x720 and up
// alone with the smaller ones grouped; frames of 1920x1080 and up alone. Phase 1 runs
// kGroupRounds passes over them (the first not scored).
struct Grouping
{
    uint64_t group, single;
};
const Grouping kGroupCand[ 4 ] = { { 0ull, 0ull }, { 4ull << 20, 0ull }, { 8ull << 20, 512ull << 10 }, { 8ull << 20, 2000000ull } };
constexpr int  kGroupRounds    = 2;

struct Tuner
{
    bool                 settled = false;
    int                  phase   = 0;   // 0: launch candidates, 1: group sizes
    int                  step    = 0;   // tuning steps taken in the phase
    std::vector< Probe > probes;
};

// Candidates of a launch kind (64x4 never won on GB300 and is left to rgdn_batch_set_config;
// anti-firefly keeps 32x8, its shared-memory tile is laid out for it):
//   temporal:  persistent 32x8 and 16x16; one 32x4 tile per 128-thread block (occ 7)
//   variance:  persistent 32x8 and 16x16; one 32x8 tile per 256-thread block (occ 7)
//   a-trous:   persistent 32x8 and 16x16 at 3 blocks per SM, one 32x4 tile per block, 32x8 at 4;
//              for the first iteration also the fusion depth 2 (kOccPair): iterations 0 and 1
//              in one launch of one 32x8 tile per block, scored against the best first and
//              second iterations together
constexpr int kOccPair = 6;
int n_candidates( int kind )
{
    return kind == BS_ATROUS0 ? 5 : kind > BS_ATROUS0 ? 4 : ( kind == BS_TEMPORAL || kind == BS_VARIANCE ) ? 3
         : 1;
}
int max_candidates() { return 5; }
void candidate( int kind, int c, int& shape, int& occ )
{
    static const int atrousShape[ 5 ] = { RGDN_TILE_32X8, RGDN_TILE_16X16, RGDN_TILE_32X4, RGDN_TILE_32X8, RGDN_TILE_32X8 };
    static const int atrousOcc[ 5 ]   = { 3, 3, 7, 4, kOccPair };
    if( kind >= BS_ATROUS0 )
    {
        const int k = c % n_candidates( kind );
        shape       = atrousShape[ k ];
        occ         = atrousOcc[ k ];
    }
    else if( kind == BS_TEMPORAL )
    {
        shape = c % 3 == 2 ? (int)RGDN_TILE_32X4 : c % 3;
        occ   = c % 3 == 2 ? 7 : 0;
    }
    else if( kind == BS_VARIANCE )
    {
        shape = c % 3 == 2 ? (int)RGDN_TILE_32X8_PER_BLOCK : c % 3;
        occ   = c % 3 == 2 ? 7 : 0;
    }
    else
    {
        shape = ( kind == BS_GRADIENT || kind == BS_ANTI_FIREFLY ) ? 0 : c % 2;
        occ   = 0;
    }
}

struct Pending
{
    int         stage, iter;
    cudaEvent_t a, b;
};

int ceil_div( int a, int b ) { return ( a + b - 1 ) / b; }

}  // namespace

// one-frame groups run on the caller's stream and kSideLanes more: on GB300 the 32-stream mix
// ran 4152 Mpix/s with one side lane, 4199-4203 with two and 4204-4207 with three
constexpr int kSideLanes = 2;

struct BatchExec
{
    int                        device = 0, sms = 0;
    cudaStream_t               capture = nullptr;   // private stream the graphs are captured on
    cudaStream_t               side[ kSideLanes ] = {};   // lanes of one-frame groups beside the caller's
    cudaEvent_t                fork = nullptr, join[ kSideLanes ] = {};
    cudaGraphExec_t            exec[ BATCH_SLOTS ] = {};
    GraphKey                   key[ BATCH_SLOTS ];
    Config                     cfg[ 4 ];
    Tuner                      tuner[ 4 ];
    int                        bps[ 4 ][ RGDN_STAGE_COUNT ][ 8 ];   // resident blocks per SM by variant, -1 = unknown
    bool                       timing = false;
    std::vector< Pending >     pending;
    std::vector< cudaEvent_t > eventPool;
};

namespace
{

cudaEvent_t take_event( BatchExec& ex )
{
    if( !ex.eventPool.empty() )
    {
        cudaEvent_t e = ex.eventPool.back();
        ex.eventPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    return cudaEventCreate( &e ) == cudaSuccess ? e : nullptr;
}

int blocks_per_sm( BatchExec& ex, uint32_t storage, int stage, int occ )
{
    int& v = ex.bps[ storage ][ stage ][ occ ];
    if( v < 0 )
    {
        BpsFn f = bps_fn( storage, stage );
        v       = f ? f( stage | ( occ << 10 ) ) : 0;
    }
    return v;
}

BatchExec* create_exec( int device )
{
    BatchExec* ex = new( std::nothrow ) BatchExec();
    if( !ex ) return nullptr;
    ex->device = device;
    bool ok    = cudaDeviceGetAttribute( &ex->sms, cudaDevAttrMultiProcessorCount, device ) == cudaSuccess && ex->sms > 0;
    ok         = ok && cudaStreamCreateWithFlags( &ex->capture, cudaStreamNonBlocking ) == cudaSuccess;
    for( int l = 0; l < kSideLanes; l++ )
    {
        ok = ok && cudaStreamCreateWithFlags( &ex->side[ l ], cudaStreamNonBlocking ) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags( &ex->join[ l ], cudaEventDisableTiming ) == cudaSuccess;
    }
    ok         = ok && cudaEventCreateWithFlags( &ex->fork, cudaEventDisableTiming ) == cudaSuccess;
    for( int s = 0; s < 4; s++ )
    {
        for( int k = 0; k < BS_COUNT; k++ )
        {
            ex->cfg[ s ].shape[ k ] = 0;
            ex->cfg[ s ].occ[ k ]   = k >= BS_ATROUS0 ? 3 : 0;
        }
        ex->cfg[ s ].graphs      = true;
        ex->cfg[ s ].groupPixels  = kGroupCand[ 2 ].group;
        ex->cfg[ s ].singlePixels = kGroupCand[ 2 ].single;
        for( int st = 0; st < RGDN_STAGE_COUNT; st++ )
            for( int o = 0; o < 8; o++ ) ex->bps[ s ][ st ][ o ] = -1;
    }
    if( !ok )
    {
        batch_exec_free( ex );
        return nullptr;
    }
    return ex;
}

}  // namespace

void batch_exec_free( BatchExec* ex )
{
    if( !ex ) return;
    for( int s = 0; s < BATCH_SLOTS; s++ )
        if( ex->exec[ s ] ) cudaGraphExecDestroy( ex->exec[ s ] );
    for( auto& t : ex->tuner )
        for( auto& p : t.probes )
        {
            cudaEventSynchronize( p.b );
            cudaEventDestroy( p.a );
            cudaEventDestroy( p.b );
        }
    for( auto& p : ex->pending )
    {
        cudaEventSynchronize( p.b );
        cudaEventDestroy( p.a );
        cudaEventDestroy( p.b );
    }
    for( cudaEvent_t e : ex->eventPool ) cudaEventDestroy( e );
    if( ex->capture ) cudaStreamDestroy( ex->capture );
    for( int l = 0; l < kSideLanes; l++ )
    {
        if( ex->side[ l ] ) cudaStreamDestroy( ex->side[ l ] );
        if( ex->join[ l ] ) cudaEventDestroy( ex->join[ l ] );
    }
    if( ex->fork ) cudaEventDestroy( ex->fork );
    delete ex;
}

namespace
{

// Enqueues the step's table copies and launches on `cs` (the captured stream when capturing):
// the stage sequence once per group. pixels[g][kind]: the pixels of group g's launch of a kind.
rgdn_status enqueue_step( rgdn_context* c, BatchExec& ex, DeviceSlots& ds, int slot, const GraphKey& key, const rgdn_job* jobs,
                          const double ( *pixels )[ BS_COUNT ], int n, int tuneCand, cudaStream_t cs, bool capturing )
{
    const uint32_t st    = (uint32_t)key.storage;
    const size_t   bytes = capturing ? sizeof( BatchConst ) : table_bytes( n );
    bool           table = false;   // a group on the batched kernels reads the table
    for( int gi = 0; gi < key.ng; gi++ ) table = table || !key.g[ gi ].single;
    if( table && ( cudaMemcpyAsync( ds.mode[ st ][ slot ], ds.host[ slot ], bytes, cudaMemcpyHostToDevice, cs ) != cudaSuccess ||
                   cudaMemcpyAsync( ds.fast[ st ][ slot ], ds.host[ slot ], bytes, cudaMemcpyHostToDevice, cs ) != cudaSuccess ) )
        return RGDN_DEVICE_ERROR;
    Tuner&     tu     = ex.tuner[ st ];
    const bool tuning = !capturing && !tu.settled && tu.phase == 0;
    const bool user   = !capturing && ex.timing;

    // One-frame groups take turns on up to 1 + kSideLanes lanes, cs and side streams: the frames
    // are of different camera streams, so one frame's kernels fill the SMs the others leave idle
    // at their launch boundaries and wave tails. The side lanes start after everything before the
    // step on cs and cs waits for them at the end (timed steps keep one lane, so each event
    // brackets one frame).
    int  singles = 0;
    bool forked  = false;
    for( int gi = 0; gi < key.ng; gi++ ) singles += key.g[ gi ].single;
    const bool twoLanes = singles > 1 && !user && !capturing;
    const int lanes = twoLanes ? std::min( singles, 1 + kSideLanes ) : 1;
    // frames side by side keep no persisting L2 window (rgdn_api.cu, run_denoise_fused), and
    // unless the step is one frame alone, the lines earlier frames left persisting return to
    // normal first, so the whole L2 serves the step
    struct NoWindow
    {
        explicit NoWindow( bool on ) { tl_l2windowOff = on; }
        ~NoWindow() { tl_l2windowOff = false; }
    } noWindow( lanes > 1 );
    const bool alone = key.ng == 1 && key.g[ 0 ].single;   // one frame, alone on the GPU
    if( !alone && c->l2Dirty.exchange( false ) ) cudaCtxResetPersistingL2Cache();
    if( twoLanes )
    {
        if( cudaEventRecord( ex.fork, cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
        for( int l = 0; l + 1 < lanes; l++ )
            if( cudaStreamWaitEvent( ex.side[ l ], ex.fork, 0 ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
        forked = true;
    }
    int nthSingle = 0;
    for( int gi = 0; gi < key.ng; gi++ )
    {
        const GroupKey& gk = key.g[ gi ];
        if( gk.single )
        {
            // one frame: the single-frame kernels, with its arguments as kernel parameters
            const rgdn_job&    jb   = jobs[ gk.j0 ];
            const int          li   = twoLanes ? nthSingle++ % lanes : 0;
            const cudaStream_t lane = li ? ex.side[ li - 1 ] : cs;
            cudaEvent_t        ua = nullptr, ub = nullptr;
            if( user )
            {
                ua = take_event( ex );
                ub = take_event( ex );
                if( !ua || !ub ) return RGDN_DEVICE_ERROR;
                cudaEventRecord( ua, lane );
            }
            rgdn_status r = run_denoise( jb.stream, jb.frameIndex, jb.params, lane );
            if( r == RGDN_SUCCESS ) r = run_exposure( jb.stream, jb.frameIndex, jb.params, lane );
            if( user )
            {
                cudaEventRecord( ub, lane );
                ex.pending.push_back( { (int)RGDN_BATCH_SINGLE_FRAME_GROUP, 0, ua, ub } );
            }
            if( r != RGDN_SUCCESS ) return r;
            continue;
        }
        const int sarg = slot | ( gk.j0 << 8 ) | ( gk.j1 << 16 );
        auto run = [ & ]( int kind, int stage, int arg, int shape, int occ, int cand ) -> rgdn_status {
            BatchLauncher L = batch_launcher( st, stage );
            if( !L ) return RGDN_INTERNAL_ERROR;
            // persistent launches: resident blocks per SM x SMs; one-tile-per-block launches: the
            // group's tiles; the luminance average: one block per frame
            const int grid = stage == RGDN_STAGE_LUMINANCE_AVG ? gk.j1 - gk.j0
                           : ( occ == 7 || occ == kOccPair )   ? gk.tiles[ kind ]
                                                               : blocks_per_sm( ex, st, stage, occ ) * ex.sms;
            if( grid <= 0 ) return RGDN_DEVICE_ERROR;
            cudaEvent_t ta = nullptr, tb = nullptr, ua = nullptr, ub = nullptr;
            if( tuning && kind >= 0 )
            {
                ta = take_event( ex );
                tb = take_event( ex );
                if( !ta || !tb ) return RGDN_DEVICE_ERROR;
                cudaEventRecord( ta, cs );
            }
            if( user )
            {
                ua = take_event( ex );
                ub = take_event( ex );
                if( !ua || !ub ) return RGDN_DEVICE_ERROR;
                cudaEventRecord( ua, cs );
            }
            const cudaError_t e = L( stage, arg, sarg, kShapes[ shape ], grid, cs );
            if( user )
            {
                cudaEventRecord( ub, cs );
                ex.pending.push_back( { stage, arg & 0xff, ua, ub } );
            }
            if( ta )
            {
                cudaEventRecord( tb, cs );
                tu.probes.push_back( { kind, cand, pixels[ gi ][ kind ], ta, tb, tuneCand >= max_candidates() } );
            }
            if( !capturing ) c->launches.fetch_add( 1, std::memory_order_relaxed );
            return cuda_status( e );
        };

        rgdn_status r;
        if( gk.anyGrad )
        {
            if( ( r = run( -1, RGDN_STAGE_GRADIENT_SAMPLES, 0, 0, 0, 0 ) ) != RGDN_SUCCESS ) return r;
            for( int i = 0; i < 4; i++ )
                if( ( r = run( -1, RGDN_STAGE_GRADIENT_ATROUS, i, 0, 0, 0 ) ) != RGDN_SUCCESS ) return r;
        }
        const int stages[ 3 ] = { RGDN_STAGE_TEMPORAL_ACCUMULATION, RGDN_STAGE_ANTI_FIREFLY, RGDN_STAGE_VARIANCE_ESTIMATION };
        for( int k = 0; k < 3; k++ )
        {
            const int kind = BS_TEMPORAL + k;
            const int arg  = k == 0 ? ( gk.gpm << 8 ) | ( key.occ[ kind ] << 10 ) : ( key.occ[ kind ] << 10 );
            if( ( r = run( kind, stages[ k ], arg, key.shape[ kind ], key.occ[ kind ], tuneCand % n_candidates( kind ) ) ) != RGDN_SUCCESS )
                return r;
        }
        for( int i = 0; i < gk.maxIter; i++ )
        {
            const int kind = BS_ATROUS0 + i;
            // fusion depth 2: the first launch ran iterations 0 and 1
            if( i == 1 && key.occ[ BS_ATROUS0 ] == kOccPair ) continue;
            const int arg = i | ( gk.hm[ i ] << 8 ) | ( key.occ[ kind ] << 10 );
            if( ( r = run( kind, RGDN_STAGE_ATROUS, arg, key.shape[ kind ], key.occ[ kind ], tuneCand % n_candidates( kind ) ) ) !=
                RGDN_SUCCESS )
                return r;
        }
        if( ( r = run( -1, RGDN_STAGE_LUMINANCE_AVG, 0, 0, 0, 0 ) ) != RGDN_SUCCESS ) return r;
    }
    if( forked )
        for( int l = 0; l + 1 < lanes; l++ )
            if( cudaEventRecord( ex.join[ l ], ex.side[ l ] ) != cudaSuccess || cudaStreamWaitEvent( cs, ex.join[ l ], 0 ) != cudaSuccess )
                return RGDN_DEVICE_ERROR;
    return RGDN_SUCCESS;
}

int kernels_in( const GraphKey& key )
{
    int k = 0;
    for( int gi = 0; gi < key.ng; gi++ )
    {
        const GroupKey& gk = key.g[ gi ];
        k += ( gk.anyGrad ? 5 : 0 ) + 3 + gk.maxIter - ( key.occ[ BS_ATROUS0 ] == kOccPair && gk.maxIter >= 2 ? 1 : 0 ) + 1;
    }
    return k;
}

// Sums the scored probes' device time and pixels by kind * stride + candidate (kind -2, a whole
// step: by candidate) and returns their events to the pool.
rgdn_status collect_probes( BatchExec& ex, Tuner& tu, std::vector< double >& ms, std::vector< double >& px, int stride )
{
    rgdn_status r = RGDN_SUCCESS;
    for( auto& p : tu.probes )
    {
        float t = 0.0f;
        if( cudaEventSynchronize( p.b ) != cudaSuccess || cudaEventElapsedTime( &t, p.a, p.b ) != cudaSuccess ) r = RGDN_DEVICE_ERROR;
        else if( p.scored && p.pixels > 0.0 )
        {
            const size_t k = (size_t)( p.kind < 0 ? 0 : p.kind * stride ) + (size_t)p.cand;
            if( k < ms.size() )
            {
                ms[ k ] += t;
                px[ k ] += p.pixels;
            }
        }
        ex.eventPool.push_back( p.a );
        ex.eventPool.push_back( p.b );
    }
    tu.probes.clear();
    return r;
}

// Picks the fastest candidate of every launch kind from the tuning steps' probes.
rgdn_status settle( BatchExec& ex, uint32_t st )
{
    Tuner&                tu = ex.tuner[ st ];
    std::vector< double > ms( BS_COUNT * max_candidates(), 0.0 ), px( BS_COUNT * max_candidates(), 0.0 );
    rgdn_status           r = collect_probes( ex, tu, ms, px, max_candidates() );
    // time per pixel of each (kind, candidate) over its scored launches (all groups, all rounds)
    std::vector< double > best( BS_COUNT * max_candidates(), 1e30 );
    for( size_t k = 0; k < best.size(); k++ )
        if( px[ k ] > 0.0 ) best[ k ] = ms[ k ] / px[ k ];
    int bestOf[ BS_COUNT ] = {};
    for( int kind = BS_TEMPORAL; kind < BS_COUNT; kind++ )
    {
        // the first iteration's single-launch candidates; the fused pair is weighed below
        const int nc    = kind == BS_ATROUS0 ? n_candidates( kind ) - 1 : n_candidates( kind );
        int       bestC = 0;
        for( int cnd = 1; cnd < nc; cnd++ )
            if( best[ kind * max_candidates() + cnd ] < best[ kind * max_candidates() + bestC ] ) bestC = cnd;
        bestOf[ kind ] = bestC;
        // kinds no tuning step ran (more iterations later) keep their configuration
        if( best[ kind * max_candidates() + bestC ] >= 1e30 ) continue;
        candidate( kind, bestC, ex.cfg[ st ].shape[ kind ], ex.cfg[ st ].occ[ kind ] );
    }
    // fusion depth 2 when the pair beats the best first and second iterations together
    const double pair = best[ BS_ATROUS0 * max_candidates() + 4 ];
    const double sep  = best[ BS_ATROUS0 * max_candidates() + bestOf[ BS_ATROUS0 ] ] +
                       best[ ( BS_ATROUS0 + 1 ) * max_candidates() + bestOf[ BS_ATROUS0 + 1 ] ];
    if( pair < 1e30 && sep < 1e30 && pair < sep ) candidate( BS_ATROUS0, 4, ex.cfg[ st ].shape[ BS_ATROUS0 ], ex.cfg[ st ].occ[ BS_ATROUS0 ] );
    // next: the group sizes, as whole steps
    tu.phase = 1;
    tu.step  = 0;
    return r;
}

// Picks the fastest group size from the whole-step probes of the second phase.
rgdn_status settle_groups( BatchExec& ex, uint32_t st )
{
    Tuner&                tu = ex.tuner[ st ];
    std::vector< double > ms( 4, 0.0 ), px( 4, 0.0 );
    rgdn_status           r    = collect_probes( ex, tu, ms, px, 4 );
    int                   best = -1;
    for( int k = 0; k < 4; k++ )
        if( px[ k ] > 0.0 && ( best < 0 || ms[ k ] / px[ k ] < ms[ best ] / px[ best ] ) ) best = k;
    if( best >= 0 )
    {
        ex.cfg[ st ].groupPixels  = kGroupCand[ best ].group;
        ex.cfg[ st ].singlePixels = kGroupCand[ best ].single;
    }
    tu.settled = true;
    return r;
}

bool batchable( const rgdn_job& j )
{
    return !( j.params->flags & ( RGDN_FLAG_PLAIN | RGDN_FLAG_EXACT_MATH | RGDN_FLAG_TMA_STAGING ) );
}

// One step over jobs[0..n) (distinct streams, one storage mode, all batchable).
rgdn_status run_step( rgdn_context* c, BatchExec& ex, const rgdn_job* jobs, int n, cudaStream_t cs )
{
    const uint32_t st = jobs[ 0 ].stream->storage;
    if( ex.device < 0 || ex.device >= kMaxDevices ) return RGDN_DEVICE_ERROR;
    DeviceSlots&                  ds = g_slots[ ex.device ];
    std::lock_guard< std::mutex > g( ds.m );
    if( !slots_ready( ds ) ) return RGDN_DEVICE_ERROR;
    const int slot = ds.next;
    ds.next        = ( ds.next + 1 ) % BATCH_SLOTS;
    if( ds.used[ slot ] )
    {
        // the slot's previous step must be done with its constant slot and host table
        if( cudaEventSynchronize( ds.done[ slot ] ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
        ds.used[ slot ] = false;
    }
    Tuner&     tu      = ex.tuner[ st ];
    const bool tuning  = !tu.settled;
    const bool tuneLk  = tuning && tu.phase == 0;   // launch candidates
    const bool tuneGrp = tuning && tu.phase == 1;   // group sizes
    int        tcand   = tu.step;
    Config     cfg     = ex.cfg[ st ];
    if( tuneLk )
        for( int kind = BS_TEMPORAL; kind < BS_COUNT; kind++ ) candidate( kind, tcand % n_candidates( kind ), cfg.shape[ kind ], cfg.occ[ kind ] );
    if( tuneGrp )
    {
        cfg.groupPixels  = kGroupCand[ tcand % 4 ].group;
        cfg.singlePixels = kGroupCand[ tcand % 4 ].single;
    }
    // the fused first two iterations need every frame of the step to run at least three
    int minIter = MAX_ATROUS_ITERATIONS;
    for( int k = 0; k < n; k++ ) minIter = std::min( minIter, jobs[ k ].params->atrousIterations ? (int)jobs[ k ].params->atrousIterations : 4 );
    if( cfg.occ[ BS_ATROUS0 ] == kOccPair && minIter < 3 )
    {
        candidate( BS_ATROUS0, 0, cfg.shape[ BS_ATROUS0 ], cfg.occ[ BS_ATROUS0 ] );
        // not scored as the pair: this tuning step counts as a warm-up step
        if( tuneLk ) tcand = tcand % max_candidates();
    }

    BatchConst* tab = ds.host[ slot ];
    memset( tab, 0, offsetof( BatchConst, jobs ) );
    tab->n = n;
    GraphKey key;
    memset( &key, 0, sizeof( key ) );
    key.storage = (int)st;
    // groups: consecutive frames while their pixels stay within the group size; a frame of at
    // least singlePixels pixels alone
    bool anySingle           = false;
    bool single[ MAX_BATCH ] = {};
    {
        uint64_t acc = 0;
        int      j0  = 0;
        auto     close = [ & ]( int j1, bool alone ) {
            key.g[ key.ng ].j0     = j0;
            key.g[ key.ng ].j1     = j1;
            key.g[ key.ng++ ].single = alone ? 1 : 0;
            if( alone )
            {
                single[ j0 ] = true;
                anySingle    = true;
            }
            j0  = j1;
            acc = 0;
        };
        for( int k = 0; k < n; k++ )
        {
            const uint64_t px = (uint64_t)jobs[ k ].stream->W * jobs[ k ].stream->H;
            if( cfg.singlePixels && px >= cfg.singlePixels )
            {
                if( k > j0 ) close( k, false );
                close( k + 1, true );
                continue;
            }
            if( k > j0 && cfg.groupPixels && acc + px > cfg.groupPixels ) close( k, false );
            acc += px;
        }
        if( n > j0 ) close( n, false );
    }
    for( int k = 0; k < n; k++ )
    {
        if( single[ k ] )
        {
            // the single-frame path fills its own arguments and keeps its stream's state
            memset( &tab->jobs[ k ], 0, sizeof( FrameArgs ) );
            tab->jobFlags[ k ] = 0;
            continue;
        }
        rgdn_stream*             s  = jobs[ k ].stream;
        const uint32_t           fi = jobs[ k ].frameIndex;
        const rgdn_frame_params* p  = jobs[ k ].params;
        rgdn_status              r  = ensure_bin_lut( s, p, cs );
        if( r != RGDN_SUCCESS ) return r;
        fill_args( s, fi, p, tab->jobs[ k ] );
        const bool gp      = s->geomValid[ fi ^ 1u ];
        tab->jobFlags[ k ] = ( gp ? BATCH_JOB_GEOM_PREV : 0u ) | ( s->histPending ? BATCH_JOB_CLEAR_HIST : 0u );
        s->geomValid[ fi ] = true;
        s->histPending     = false;
    }
    // tile tables (numbered over the whole step) and pixels per group and launch kind
    double pixels[ MAX_BATCH ][ BS_COUNT ] = {};
    double stepPixels                      = 0.0;
    for( int kind = 0; kind < BS_COUNT; kind++ )
    {
        const dim3 sh  = kind == BS_ANTI_FIREFLY ? dim3( 32, af_tile_rows( (int)st ) ) : kShapes[ kind == BS_GRADIENT ? 0 : cfg.shape[ kind ] ];
        int        acc = 0;
        for( int gi = 0; gi < key.ng; gi++ )
        {
            GroupKey& gk = key.g[ gi ];
            for( int k = gk.j0; k < gk.j1; k++ )
            {
                tab->start[ kind ][ k ] = acc;
                const Uniform& u        = tab->jobs[ k ].u;
                bool           runs;
                if( single[ k ] ) runs = false;
                else if( kind == BS_GRADIENT ) runs = !( u.flags & RGDN_FLAG_SKIP_GRADIENTS );
                else if( kind >= BS_ATROUS0 ) runs = (int)u.niter > kind - BS_ATROUS0;
                else runs = true;
                if( !runs ) continue;
                const int w = kind == BS_GRADIENT ? u.GW : u.W, h = kind == BS_GRADIENT ? u.GH : u.H;
                acc += ceil_div( w, (int)sh.x ) * ceil_div( h, (int)sh.y );
                pixels[ gi ][ kind ] += (double)w * h;
            }
            if( kind != BS_GRADIENT && ( cfg.occ[ kind ] == 7 || cfg.occ[ kind ] == kOccPair ) )
                gk.tiles[ kind ] = acc - tab->start[ kind ][ gk.j0 ];
        }
        tab->start[ kind ][ n ] = acc;
    }
    for( int k = 0; k < n; k++ ) stepPixels += (double)jobs[ k ].stream->W * jobs[ k ].stream->H;
    for( int gi = 0; gi < key.ng; gi++ )
    {
        GroupKey& gk      = key.g[ gi ];
        int       gpValid = 0;
        if( gk.single ) continue;
        for( int k = gk.j0; k < gk.j1; k++ )
        {
            gpValid += ( tab->jobFlags[ k ] & BATCH_JOB_GEOM_PREV ) ? 1 : 0;
            gk.maxIter = std::max( gk.maxIter, (int)tab->jobs[ k ].u.niter );
            if( !( tab->jobs[ k ].u.flags & RGDN_FLAG_SKIP_GRADIENTS ) ) gk.anyGrad = 1;
        }
        gk.gpm = gpValid == 0 ? 0 : gpValid == gk.j1 - gk.j0 ? 1 : 2;
        for( int i = 0; i < gk.maxIter; i++ )
        {
            int runs = 0, last = 0;
            for( int k = gk.j0; k < gk.j1; k++ )
            {
                if( (int)tab->jobs[ k ].u.niter > i ) runs++;
                if( (int)tab->jobs[ k ].u.niter == i + 1 ) last++;
            }
            gk.hm[ i ] = last == 0 ? 0 : last == runs ? 1 : 2;
        }
    }
    for( int kind = 0; kind < BS_COUNT; kind++ )
    {
        key.shape[ kind ] = kind == BS_GRADIENT ? 0 : cfg.shape[ kind ];
        key.occ[ kind ]   = cfg.occ[ kind ];
    }

    rgdn_status r = RGDN_SUCCESS;
    // a step with a single-frame group is launched directly: that group's kernel parameters
    // change every step
    if( cfg.graphs && !tuning && !ex.timing && !anySingle )
    {
        cudaGraphExec_t& exec = ex.exec[ slot ];
        if( !exec || !same_key( ex.key[ slot ], key ) )
        {
            cudaGraph_t g = nullptr;
            if( cudaStreamBeginCapture( ex.capture, cudaStreamCaptureModeThreadLocal ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
            r             = enqueue_step( c, ex, ds, slot, key, jobs, pixels, n, 0, ex.capture, true );
            cudaError_t e = cudaStreamEndCapture( ex.capture, &g );
            if( r == RGDN_SUCCESS && e != cudaSuccess ) r = RGDN_DEVICE_ERROR;
            if( r == RGDN_SUCCESS )
            {
                if( exec )
                {
                    cudaGraphExecUpdateResultInfo info;
                    if( cudaGraphExecUpdate( exec, g, &info ) != cudaSuccess )
                    {
                        cudaGetLastError();
                        cudaGraphExecDestroy( exec );
                        exec = nullptr;
                    }
                }
                if( !exec && cudaGraphInstantiate( &exec, g, 0 ) != cudaSuccess )
                {
                    exec = nullptr;
                    r    = RGDN_DEVICE_ERROR;
                }
                ex.key[ slot ] = key;
            }
            if( g ) cudaGraphDestroy( g );
            if( r != RGDN_SUCCESS ) return r;
        }
        if( cudaGraphLaunch( exec, cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
        c->launches.fetch_add( (uint64_t)kernels_in( key ), std::memory_order_relaxed );
    }
    else
    {
        cudaEvent_t ga = nullptr, gb = nullptr;
        if( tuneGrp )
        {
            ga = take_event( ex );
            gb = take_event( ex );
            if( !ga || !gb ) return RGDN_DEVICE_ERROR;
            cudaEventRecord( ga, cs );
        }
        if( ( r = enqueue_step( c, ex, ds, slot, key, jobs, pixels, n, tcand, cs, false ) ) != RGDN_SUCCESS ) return r;
        if( ga )
        {
            cudaEventRecord( gb, cs );
            tu.probes.push_back( { -2, tcand % 4, stepPixels, ga, gb, tcand >= 4 } );
        }
    }
    // the slot's host table is read by the device only when a group ran on the batched kernels
    bool anyTable = false;
    for( int gi = 0; gi < key.ng; gi++ ) anyTable = anyTable || !key.g[ gi ].single;
    if( anyTable )
    {
        if( cudaEventRecord( ds.done[ slot ], cs ) != cudaSuccess ) return RGDN_DEVICE_ERROR;
        ds.used[ slot ] = true;
    }
    if( tuneLk && ++tu.step >= kTuneRounds * max_candidates() ) r = settle( ex, st );
    else if( tuneGrp && ++tu.step >= kGroupRounds * 4 ) r = settle_groups( ex, st );
    return r;
}

BatchExec* exec_of( rgdn_context* c )
{
    if( !c->batch ) c->batch = create_exec( c->device );
    return c->batch;
}

}  // namespace

rgdn_status batch_submit( rgdn_context* c, const rgdn_job* jobs, uint32_t n, cudaStream_t cs )
{
    std::lock_guard< std::mutex > g( c->batchMtx );
    BatchExec*                    ex = exec_of( c );
    if( !ex ) return RGDN_DEVICE_ERROR;
    uint32_t i = 0;
    while( i < n )
    {
        if( !batchable( jobs[ i ] ) )
        {
            rgdn_status r = run_denoise( jobs[ i ].stream, jobs[ i ].frameIndex, jobs[ i ].params, cs );
            if( r == RGDN_SUCCESS ) r = run_exposure( jobs[ i ].stream, jobs[ i ].frameIndex, jobs[ i ].params, cs );
            if( r != RGDN_SUCCESS ) return r;
            i++;
            continue;
        }
        // a step: consecutive batchable jobs of one storage mode on distinct streams
        uint32_t end = i;
        while( end < n && end - i < (uint32_t)MAX_BATCH && batchable( jobs[ end ] ) &&
               jobs[ end ].stream->storage == jobs[ i ].stream->storage )
        {
            bool dup = false;
            for( uint32_t k = i; k < end && !dup; k++ ) dup = jobs[ k ].stream == jobs[ end ].stream;
            if( dup ) break;
            end++;
        }
        rgdn_status r = run_step( c, *ex, jobs + i, (int)( end - i ), cs );
        if( r != RGDN_SUCCESS ) return r;
        i = end;
    }
    return RGDN_SUCCESS;
}

void batch_destroy( rgdn_context* c )
{
    std::lock_guard< std::mutex > g( c->batchMtx );
    if( c->batch && c->batch->device >= 0 && c->batch->device < kMaxDevices )
    {
        // steps of this context may still use the device's slots
        DeviceSlots&                  ds = g_slots[ c->batch->device ];
        std::lock_guard< std::mutex > gs( ds.m );
        for( int s = 0; s < BATCH_SLOTS; s++ )
            if( ds.used[ s ] ) cudaEventSynchronize( ds.done[ s ] );
    }
    batch_exec_free( c->batch );
    c->batch = nullptr;
}

rgdn_status batch_get_config( rgdn_context* c, uint32_t storage, rgdn_batch_config* out )
{
    std::lock_guard< std::mutex > g( c->batchMtx );
    BatchExec*                    ex = exec_of( c );
    if( !ex ) return RGDN_DEVICE_ERROR;
    const Config& cf = ex->cfg[ storage ];
    memset( out, 0, sizeof( *out ) );
    out->temporalTile    = (uint32_t)cf.shape[ BS_TEMPORAL ];
    out->antiFireflyTile = (uint32_t)cf.shape[ BS_ANTI_FIREFLY ];
    out->varianceTile    = (uint32_t)cf.shape[ BS_VARIANCE ];
    for( int i = 0; i < MAX_ATROUS_ITERATIONS; i++ )
    {
        out->atrousTile[ i ]        = (uint32_t)cf.shape[ BS_ATROUS0 + i ];
        out->atrousBlocksPerSM[ i ] = (uint32_t)cf.occ[ BS_ATROUS0 + i ];
    }
    out->atrousFusionDepth = cf.occ[ BS_ATROUS0 ] == kOccPair ? 2u : 1u;
    if( out->atrousFusionDepth == 2u ) out->atrousBlocksPerSM[ 0 ] = 3;   // the pair kernel's build
    out->useGraphs   = cf.graphs ? 1u : 0u;
    out->tuned       = ex->tuner[ storage ].settled ? 1u : 0u;
    out->groupPixels = cf.groupPixels;
    out->singleFramePixels = cf.singlePixels;
    return RGDN_SUCCESS;
}

rgdn_status batch_set_config( rgdn_context* c, uint32_t storage, const rgdn_batch_config* in )
{
    // 32x4 (128-thread) tiles exist for the temporal and a-trous kernels only
    auto ok_shape = []( uint32_t v ) { return v <= RGDN_TILE_64X4; };
    auto ok_shape4 = []( uint32_t v ) { return v <= RGDN_TILE_32X4; };
    if( !ok_shape4( in->temporalTile ) || !ok_shape( in->antiFireflyTile ) ||
        !( ok_shape( in->varianceTile ) || in->varianceTile == RGDN_TILE_32X8_PER_BLOCK ) )
        return RGDN_WRONG_FUNCTION_ARGUMENT;
    for( int i = 0; i < MAX_ATROUS_ITERATIONS; i++ )
    {
        const uint32_t b = in->atrousBlocksPerSM[ i ];
        if( !ok_shape4( in->atrousTile[ i ] ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
        if( in->atrousTile[ i ] == RGDN_TILE_32X4 ? ( b && b != 7 ) : ( b && ( b < 3 || b > 4 ) ) ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    }
    if( in->atrousFusionDepth > 2 ) return RGDN_WRONG_FUNCTION_ARGUMENT;
    std::lock_guard< std::mutex > g( c->batchMtx );
    BatchExec*                    ex = exec_of( c );
    if( !ex ) return RGDN_DEVICE_ERROR;
    Config& cf                  = ex->cfg[ storage ];
    cf.shape[ BS_TEMPORAL ]     = (int)in->temporalTile;
    cf.occ[ BS_TEMPORAL ]       = in->temporalTile == RGDN_TILE_32X4 ? 7 : 0;
    cf.shape[ BS_ANTI_FIREFLY ] = 0;   // the shared-memory tile is 32x8
    cf.shape[ BS_VARIANCE ]     = (int)in->varianceTile;
    cf.occ[ BS_VARIANCE ]       = in->varianceTile == RGDN_TILE_32X8_PER_BLOCK ? 7 : 0;
    for( int i = 0; i < MAX_ATROUS_ITERATIONS; i++ )
    {
        cf.shape[ BS_ATROUS0 + i ] = (int)in->atrousTile[ i ];
        cf.occ[ BS_ATROUS0 + i ]   = in->atrousTile[ i ] == RGDN_TILE_32X4 ? 7 : in->atrousBlocksPerSM[ i ] ? (int)in->atrousBlocksPerSM[ i ] : 3;
    }
    if( in->atrousFusionDepth == 2 ) candidate( BS_ATROUS0, 4, cf.shape[ BS_ATROUS0 ], cf.occ[ BS_ATROUS0 ] );
    cf.graphs      = in->useGraphs != 0;
    cf.groupPixels  = in->groupPixels;
    cf.singlePixels = in->singleFramePixels;
    Tuner& tu = ex->tuner[ storage ];
    for( auto& p : tu.probes )
    {
        cudaEventSynchronize( p.b );
        ex->eventPool.push_back( p.a );
        ex->eventPool.push_back( p.b );
    }
    tu.probes.clear();
    tu.settled = true;
    return RGDN_SUCCESS;
}

rgdn_status batch_set_timing( rgdn_context* c, bool enable )
{
    std::lock_guard< std::mutex > g( c->batchMtx );
    BatchExec*                    ex = exec_of( c );
    if( !ex ) return RGDN_DEVICE_ERROR;
    ex->timing = enable;
    return RGDN_SUCCESS;
}

rgdn_status batch_read_timing( rgdn_context* c, rgdn_stage_timing* out, uint32_t capacity, uint32_t* outCount )
{
    std::lock_guard< std::mutex > g( c->batchMtx );
    BatchExec*                    ex = exec_of( c );
    if( !ex ) return RGDN_DEVICE_ERROR;
    std::vector< rgdn_stage_timing > agg;
    rgdn_status                      r = RGDN_SUCCESS;
    for( auto& pd : ex->pending )
    {
        float ms = 0.0f;
        if( cudaEventSynchronize( pd.b ) != cudaSuccess || cudaEventElapsedTime( &ms, pd.a, pd.b ) != cudaSuccess ) r = RGDN_DEVICE_ERROR;
        auto it = std::find_if( agg.begin(), agg.end(), [ & ]( const rgdn_stage_timing& t ) {
            return t.stage == (uint32_t)pd.stage && t.iteration == (uint32_t)pd.iter;
        } );
        if( it == agg.end() ) agg.push_back( { (uint32_t)pd.stage, (uint32_t)pd.iter, 1u, ms } );
        else
        {
            it->launches++;
            it->totalMs += ms;
        }
        ex->eventPool.push_back( pd.a );
        ex->eventPool.push_back( pd.b );
    }
    ex->pending.clear();
    std::sort( agg.begin(), agg.end(), []( const rgdn_stage_timing& a, const rgdn_stage_timing& b ) {
        return a.stage != b.stage ? a.stage < b.stage : a.iteration < b.iteration;
    } );
    for( uint32_t k = 0; k < agg.size() && k < capacity; k++ ) out[ k ] = agg[ k ];
    *outCount = (uint32_t)agg.size();
    return r;
}

}  // namespace rgdn
