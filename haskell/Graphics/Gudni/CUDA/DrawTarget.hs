-----------------------------------------------------------------------------
-- |
-- Module      :  Graphics.Gudni.CUDA.DrawTarget
--
-- Headless draw targets for the CUDA raster path: the counterpart of
-- Graphics.Gudni.Interface.DrawTarget (src/Graphics/Gudni/Interface/DrawTarget.hs:
-- 29-49) without SDL or OpenGL.  The reference's target is a locked SDL texture
-- (HostBitmapTarget) or an unimplemented GL texture (GLTextureTarget,
-- OpenCL/CallKernels.hs:202-205); here the rasterizer writes either a host bitmap
-- (any caller-owned memory: an SDL texture, a file buffer) or a CUDA device buffer
-- that stays on the GPU for the next consumer (an encoder, a compositor, another
-- kernel), which is what the GL-interop target was meant to be.
--
-- Written against the library's C ABI (include/gudni_cuda.h); GHC is not part of
-- the build environment this was written in, so it is reviewed, not compiled there.
-----------------------------------------------------------------------------
module Graphics.Gudni.CUDA.DrawTarget
  ( HeadlessBuffer(..)
  , HeadlessTarget(..)
  , isHostTarget
  , targetWords
  , withHostTarget
  ) where

import Foreign.C.Types (CInt, CUInt)
import Foreign.Marshal.Array (allocaArray)
import Foreign.Ptr
import Linear (V2(..))

-- | Where the BGRA words of a frame go (one 32-bit word per pixel, row-major,
-- alpha 255, as writePixelGlobal writes them, Kernels.cl:1853-1862).
data HeadlessBuffer
    -- | Host memory of at least width*height words.  Rendered by the blocking
    -- entry points (gudni_raster_job, gudni_raster_frame).
    = HostBitmap   { hostPtr :: Ptr CUInt }
    -- | CUDA device memory of at least width*height words, allocated by the host
    -- application.  Rendered by the stream-ordered entry points
    -- (gudni_raster_job_device, gudni_raster_tiles_device); the pixels stay on the
    -- device, and the stream (a cudaStream_t, nullPtr for the context's own stream)
    -- orders whatever reads them next.
    | DeviceBitmap { devicePtr :: Ptr CUInt, streamPtr :: Ptr () }

-- | A target with its size: DrawTarget's targetArea and targetBuffer, without the
-- SDL texture.
data HeadlessTarget = HeadlessTarget
    { headlessArea   :: V2 CInt
    , headlessBuffer :: HeadlessBuffer
    }

-- | True when the pixels land in host memory (isHostBitmapTarget, DrawTarget.hs:45-49).
isHostTarget :: HeadlessTarget -> Bool
isHostTarget t = case headlessBuffer t of
    HostBitmap _ -> True
    _            -> False

-- | Words the target holds.
targetWords :: HeadlessTarget -> Int
targetWords t = let V2 w h = headlessArea t in fromIntegral w * fromIntegral h

-- | A host bitmap of the given size for the duration of an action (a frame written
-- to a file, say), released afterwards.
withHostTarget :: V2 CInt -> (HeadlessTarget -> IO a) -> IO a
withHostTarget area@(V2 w h) use =
    allocaArray (fromIntegral w * fromIntegral h) $ \p -> use (HeadlessTarget area (HostBitmap p))
