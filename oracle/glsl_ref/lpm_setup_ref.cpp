// The reference's CPU-side LPM setup, compiled from its own FidelityFX headers
// (Source/Shaders/LPM/ffx_a.h, ffx_lpm.h and LpmSetupCustom.inl, found through the include path
// that oracle/glsl_ref/build.py passes): test infrastructure for the final-composition check.
//
// ref_lpm_setup fills the 24 uvec4 control words of CmPrepareFinal.comp's LpmParams_BT block
// the way ImageComposition::SetupLpmParams does (Source/ImageComposition.cpp:343-400): A_CPU
// headers, the context form of LpmSetupOut writing ctl[i * 4 + k], and LpmSetup with
// ImageComposition's fixed arguments (709 -> 709, softGap 0, hdrMax 256, exposure 8, contrast
// 0.1, shoulder contrast 1) and the caller's saturation and crosstalk.
#include <cstdint>
#include <math.h>
#include <string.h>

#define A_CPU 1
#include "ffx_a.h"

namespace
{
// ffx_lpm.h's own LpmSetup calls this form; the context form below is the one used
void LpmSetupOut( AU1, inAU4 ) {}

void LpmSetupOut( void* pContext, AU1 i, const inAU4 value )
{
    AU1* ctl = static_cast< AU1* >( pContext );
    if( i >= 24 ) return;
    for( int k = 0; k < 4; k++ ) ctl[ i * 4 + k ] = value[ k ];
}
}

#include "ffx_lpm.h"
#include "LpmSetupCustom.inl"

extern "C" void ref_lpm_setup( const float* saturation3, const float* crosstalk3, uint32_t* ctl96 )
{
    void* pContext = ctl96;
    varAF3( saturation ) = initAF3( saturation3[ 0 ], saturation3[ 1 ], saturation3[ 2 ] );
    varAF3( crosstalk )  = initAF3( crosstalk3[ 0 ], crosstalk3[ 1 ], crosstalk3[ 2 ] );
    LpmSetup( pContext, false, LPM_CONFIG_709_709, LPM_COLORS_709_709, 0.0f, 256.0f, 8.0f, 0.1f, 1.0f, saturation,
              crosstalk );
}
