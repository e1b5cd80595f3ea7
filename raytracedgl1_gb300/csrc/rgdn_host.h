// Host-side state shared by the C ABI (rgdn_api.cu) and the batch executor (rgdn_batch.cu):
// the context and stream handles and the per-frame helpers both use.
#pragma once

#include <atomic>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <vector>

#include "rgdn_internal.h"

namespace rgdn
{
struct BatchExec;
}

// ------------------------------------------------------------------------------------------
// handles
// ------------------------------------------------------------------------------------------
struct rgdn_context
{
    int                     device = 0;
    uint64_t                budget = 0;
    uint64_t                used   = 0;
    std::mutex              mtx;
    std::set< rgdn_stream* > streams;
    float2*                 phiTab   = nullptr;   // (sin phi_j, cos phi_j)
    float2*                 thetaTab = nullptr;   // (cos theta_k, sin theta_k)
    float*                  decayTab = nullptr;   // pow(1 - k/255, 10), k = 0..255
    size_t                  l2Persist = 0;        // the L2 set aside for persisting accesses
    std::atomic< bool >     l2Dirty{ false };     // a frame marked lines persisting since the last reset
    std::atomic< uint64_t > launches{ 0 };
    std::mutex              batchMtx;              // guards `batch`
    rgdn::BatchExec*        batch = nullptr;       // created by the first batched submission
    uint32_t                magic = 0x52474443u;
};

struct PlaneSlot
{
    uint8_t* ptr[ 2 ] = { nullptr, nullptr };   // in use (own plane or a bound caller plane)
    uint8_t* own[ 2 ] = { nullptr, nullptr };   // the stream's own planes
    uint32_t w = 0, h = 0, texel = 0, format = 0;
    bool     prev = false;
};

struct rgdn_stream
{
    rgdn_context*          ctx = nullptr;
    uint32_t               W = 0, H = 0, GW = 0, GH = 0, storage = 0;
    void*                  block = nullptr;
    size_t                 bytes = 0;
    PlaneSlot              planes[ RGDN_FB_COUNT ];
    rgdn::Tonemapping*     tm     = nullptr;
    uint8_t*               binLut = nullptr;
    rgdn_reshade_scene*    rsDev  = nullptr;   // device copy of the re-shade scene (stream block)
    bool                   rsSet  = false;
    float4*                geom[ 2 ] = { nullptr, nullptr };
    bool                   geomValid[ 2 ] = { false, false };   // slot holds its frame's record
    float                  lutMin = NAN, lutMax = NAN;
    std::vector< uint8_t > hostLut;
    // per-kernel timing
    struct Pending
    {
        int         stage, iter;
        cudaEvent_t a, b;
    };
    bool                        timing = false;
    bool                        histPending = false;   // a fused denoise accumulated this frame's histogram
    // tensor maps of the TMA-staged a-trous, keyed by (plane, texel words, box width, box height)
    std::map< std::tuple< const void*, int, int, int >, CUtensorMap > tmaps;
    std::vector< Pending >      pending;
    std::vector< cudaEvent_t >  eventPool;
    uint32_t                    magic = 0x52474453u;
};

namespace rgdn
{

inline bool        valid_ctx( rgdn_context* c ) { return c && c->magic == 0x52474443u; }
inline bool        valid_stream( rgdn_stream* s ) { return s && s->magic == 0x52474453u && valid_ctx( s->ctx ); }
inline rgdn_status cuda_status( cudaError_t e ) { return e == cudaSuccess ? RGDN_SUCCESS : RGDN_DEVICE_ERROR; }

rgdn_status check_params( const rgdn_frame_params* p );
// device addresses and uniform values of stream s for frame slot fi
void        fill_args( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, FrameArgs& a );
// uploads the histogram bin table when the frame's luminance range changed
rgdn_status ensure_bin_lut( rgdn_stream* s, const rgdn_frame_params* p, cudaStream_t cs );
// one frame on one stream (rgdn_denoise / rgdn_calculate_exposure)
rgdn_status run_denoise( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, cudaStream_t cs );
rgdn_status run_exposure( rgdn_stream* s, uint32_t fi, const rgdn_frame_params* p, cudaStream_t cs );

// batch executor (rgdn_batch.cu)
rgdn_status batch_submit( rgdn_context* c, const rgdn_job* jobs, uint32_t n, cudaStream_t cs );
void        batch_destroy( rgdn_context* c );
void        batch_exec_free( BatchExec* ex );
rgdn_status batch_get_config( rgdn_context* c, uint32_t storage, rgdn_batch_config* out );
rgdn_status batch_set_config( rgdn_context* c, uint32_t storage, const rgdn_batch_config* in );
rgdn_status batch_set_timing( rgdn_context* c, bool enable );
rgdn_status batch_read_timing( rgdn_context* c, rgdn_stage_timing* out, uint32_t capacity, uint32_t* outCount );

}  // namespace rgdn
