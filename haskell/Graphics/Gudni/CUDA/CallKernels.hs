{-# LANGUAGE ForeignFunctionInterface #-}
-----------------------------------------------------------------------------
-- |
-- Module      :  Graphics.Gudni.CUDA.CallKernels
--
-- Drop-in for Graphics.Gudni.OpenCL.CallKernels (src/Graphics/Gudni/OpenCL/
-- CallKernels.hs:88-255): the same job piles, handed to the sm_103a CUDA library
-- (libgudni_cuda, include/gudni_cuda.h) instead of three OpenCL kernels.  The scene
-- API, the Raster/* serializer, the tile tree and buildRasterJobs are unchanged; the
-- records passed through are the piles they already build, byte for byte.
--
-- The cabal stanza adds `extra-libraries: gudni_cuda` with the library directory
-- gudni_gb300/_build.  GHC is not part of the build environment this was written
-- in: the module is reviewed, not compiled there, and the test suite checks every
-- foreign import below against the C prototypes (argument count, and the kind and
-- size of each argument and result).
-----------------------------------------------------------------------------
module Graphics.Gudni.CUDA.CallKernels
  ( CudaRasterizer
  , withCudaRasterizer
  , queueRasterJobsCUDA
  , queueRasterJobsHeadless
  , rasterJobCUDA
  , residentPictures
  , uploadFrameCUDA
  ) where

import Control.Exception (bracket)
import Control.Lens
import Control.Monad
import Control.Monad.IO.Class
import qualified Data.Vector.Storable as VS
import Foreign
import Foreign.C.String
import Foreign.C.Types
import Graphics.Gudni.CUDA.DrawTarget
import Graphics.Gudni.Figure.Picture (PictureUsage, PictureMemoryReference, makePictData)
import Graphics.Gudni.Figure.Space (SubSpace)
import Graphics.Gudni.Interface.DrawTarget
import Graphics.Gudni.OpenCL.CallKernels (RasterParams(..), rpDevice, rpTarget, rpGeometryState, rpSubstanceState)
import Graphics.Gudni.OpenCL.Rasterizer
import Graphics.Gudni.Raster.Job
import Graphics.Gudni.Raster.Serialize
import Graphics.Gudni.Raster.ShapeInfo
import Graphics.Gudni.Raster.TileTree (adjustedLog)
import Graphics.Gudni.Util.Pile
import Linear (V2(..))

data GudniCtx
newtype CudaRasterizer = CudaRasterizer (Ptr GudniCtx)

-- | gudni_spec (include/gudni_cuda.h): seven 4-byte integers and the stochastic
-- factor, in the order of the RasterSpec fields and cppDefines (Setup.hs:45-64).
data GudniSpec = GudniSpec CInt CInt CInt CInt CInt CInt CInt CFloat
instance Storable GudniSpec where
  sizeOf _ = 32
  alignment _ = 4
  peek _ = error "GudniSpec is write-only"
  poke p (GudniSpec a b c d e f g h) = do
    pokeByteOff p 0 a; pokeByteOff p 4 b; pokeByteOff p 8 c; pokeByteOff p 12 d
    pokeByteOff p 16 e; pokeByteOff p 20 f; pokeByteOff p 24 g; pokeByteOff p 28 h

-- The context, its errors, and the per-frame uploads (setupOpenCL, BuffersInCommon).
foreign import ccall safe "gudni_create"  c_create  :: Ptr GudniSpec -> CInt -> IO (Ptr GudniCtx)
foreign import ccall safe "gudni_destroy" c_destroy :: Ptr GudniCtx -> IO ()
foreign import ccall safe "gudni_last_error" c_lastError :: Ptr GudniCtx -> IO CString
foreign import ccall safe "gudni_sync_status" c_syncStatus :: Ptr GudniCtx -> IO CInt
foreign import ccall safe "gudni_upload_common"
  c_uploadCommon :: Ptr GudniCtx -> Ptr CChar -> CSize -> Ptr CFloat -> CSize -> Ptr Word8 -> CSize
                 -> Ptr () -> CSize -> Ptr () -> CSize -> Ptr CFloat -> IO CInt
foreign import ccall safe "gudni_upload_pictures"
  c_uploadPictures :: Ptr GudniCtx -> Ptr Word8 -> CSize -> IO CInt
foreign import ccall safe "gudni_upload_random_field"
  c_uploadRandomField :: Ptr GudniCtx -> Ptr CFloat -> IO CInt
foreign import ccall safe "gudni_upload_frame"
  c_uploadFrame :: Ptr GudniCtx -> Ptr CChar -> CSize -> Ptr CFloat -> CSize -> Ptr () -> CSize
                -> Ptr () -> CSize -> IO CInt

-- One RasterJob (generateCall), host or device output.
foreign import ccall safe "gudni_raster_job"
  c_rasterJob :: Ptr GudniCtx -> Ptr () -> CSize -> Ptr () -> CSize -> CInt -> CInt -> CInt -> CInt
              -> CInt -> CInt -> Ptr CFloat -> Ptr CUInt -> IO CInt
foreign import ccall safe "gudni_raster_job_device"
  c_rasterJobDevice :: Ptr GudniCtx -> Ptr () -> CSize -> Ptr () -> CSize -> CInt -> CInt -> CInt -> CInt
                    -> CInt -> CInt -> Ptr CFloat -> Ptr CUInt -> Ptr () -> IO CInt
foreign import ccall safe "gudni_raster_tiles_device"
  c_rasterTilesDevice :: Ptr GudniCtx -> Ptr () -> CSize -> Ptr () -> Ptr Int32 -> CSize -> CInt -> CInt
                      -> CInt -> CInt -> Ptr CFloat -> Ptr Word32 -> Ptr () -> IO CInt

-- The serializer on the device (no reference counterpart; a flattened scene in,
-- the frame's piles on the device out).
foreign import ccall safe "gudni_serialize_device"
  c_serializeDevice :: Ptr GudniCtx -> Ptr () -> CInt -> Ptr () -> IO CInt

-- The batched and adjoint forms (no reference counterpart).
foreign import ccall safe "gudni_batch_upload"
  c_batchUpload :: Ptr GudniCtx -> Ptr () -> CSize -> Ptr CFloat -> CSize -> Ptr Word8 -> CSize
                -> Ptr () -> CSize -> Ptr () -> CSize -> Ptr () -> CSize -> Ptr () -> Ptr Int32
                -> Ptr CFloat -> CSize -> Ptr () -> CSize -> CSize -> IO CInt
foreign import ccall safe "gudni_batch_render"   c_batchRender   :: Ptr GudniCtx -> CInt -> Ptr () -> IO CInt
foreign import ccall safe "gudni_batch_download" c_batchDownload :: Ptr GudniCtx -> Ptr Word32 -> IO CInt
foreign import ccall safe "gudni_batch_adjoint"
  c_batchAdjoint :: Ptr GudniCtx -> Ptr CFloat -> Ptr CFloat -> Ptr CFloat -> Ptr CFloat -> Ptr () -> IO CInt
foreign import ccall safe "gudni_adjoint_tiles_device"
  c_adjointTilesDevice :: Ptr GudniCtx -> Ptr () -> CSize -> Ptr () -> Ptr Int32 -> CSize -> CInt -> CInt
                       -> CInt -> Ptr CFloat -> Ptr CFloat -> Ptr CFloat -> Ptr CFloat -> Ptr CFloat
                       -> Ptr () -> IO CInt

check :: Ptr GudniCtx -> CInt -> IO ()
check ctx rc = unless (rc == 0) $ c_lastError ctx >>= peekCString >>= ioError . userError

-- | setupOpenCL's counterpart (Setup.hs:102-147): one context on CUDA device 0, with
-- the RasterSpec the host already determined (MAXSHAPE and SHAPESTACKSECTIONS from
-- Raster/Constants.hs, as cppDefines injects them; STOCHASTIC_FACTOR 0).
withCudaRasterizer :: RasterSpec -> Int -> Int -> (CudaRasterizer -> IO a) -> IO a
withCudaRasterizer spec maxShape stackSections use =
  bracket create c_destroy (use . CudaRasterizer)
  where
    create = with (GudniSpec (fi (spec ^. specMaxTileSize)) (fi (spec ^. specThreadsPerTile))
                             (fi (spec ^. specMaxStrandsPerTile)) (fi (spec ^. specMaxTilesPerCall))
                             (fi (spec ^. specMaxThresholds)) (fi maxShape) (fi stackSections) 0) $ \p -> do
      ctx <- c_create p 0
      when (ctx == nullPtr) $ c_lastError nullPtr >>= peekCString >>= ioError . userError
      return ctx
    fi :: (Integral a, Num b) => a -> b
    fi = fromIntegral

-- | In place of generateCall (CallKernels.hs:88-179): the job's piles go to the GPU
-- as they are; the library owns the per-job scratch and reports overflow as an error.
rasterJobCUDA :: CudaRasterizer -> RasterJob -> V2 CInt -> CInt -> CInt -> CInt
              -> Ptr CFloat -> Ptr CUInt -> IO ()
rasterJobCUDA (CudaRasterizer ctx) job (V2 w h) computeDepth frame jobIndex background out = do
  let shapes = job ^. rJShapePile
      tiles  = job ^. rJTilePile
  check ctx =<< c_rasterJob ctx (castPtr (_pileData shapes)) (fromIntegral (shapes ^. pileSize))
                               (castPtr (_pileData tiles))  (fromIntegral (tiles  ^. pileSize))
                               (fromIntegral (job ^. rJColumnAllocation)) w h computeDepth frame jobIndex
                               background out

-- | The job into a device buffer, enqueued on the target's stream; errors found on
-- the device surface at the next gudni_sync_status.
rasterJobDevice :: CudaRasterizer -> RasterJob -> V2 CInt -> CInt -> CInt -> CInt
                -> Ptr CFloat -> Ptr CUInt -> Ptr () -> IO ()
rasterJobDevice (CudaRasterizer ctx) job (V2 w h) computeDepth frame jobIndex background out stream = do
  let shapes = job ^. rJShapePile
      tiles  = job ^. rJTilePile
  check ctx =<< c_rasterJobDevice ctx (castPtr (_pileData shapes)) (fromIntegral (shapes ^. pileSize))
                                     (castPtr (_pileData tiles))  (fromIntegral (tiles  ^. pileSize))
                                     (fromIntegral (job ^. rJColumnAllocation)) w h computeDepth frame
                                     jobIndex background out stream

-- | BuffersInCommon (CallKernels.hs:208-240) as one upload: the geometry pile, the
-- substance pile, the makePictData piles and the random field.
uploadCommon :: CudaRasterizer -> RasterParams token -> IO ()
uploadCommon (CudaRasterizer ctx) params = do
  let geo  = params ^. rpGeometryState . geoGeometryPile
      subs = params ^. rpSubstanceState . suSubstancePile
  (pictData, pictUsage) <- makePictData (params ^. rpSubstanceState . suPictureMapping)
                                        (params ^. rpSubstanceState . suPictureUsages)
  VS.unsafeWith (params ^. rpGeometryState . geoRandomField) $ \randoms ->
    check ctx =<< c_uploadCommon ctx (_pileData geo) (fromIntegral (geo ^. pileSize))
                                     (castPtr (_pileData subs)) (fromIntegral (subs ^. pileSize))
                                     (_pileData pictData) (fromIntegral (pictData ^. pileSize))
                                     (castPtr (_pileData pictUsage)) (fromIntegral (pictUsage ^. pileSize))
                                     nullPtr 0 (castPtr randoms)

computeDepthOf :: RasterParams token -> CInt
computeDepthOf params =
  adjustedLog (fromIntegral (params ^. rpDevice . rasterSpec . specThreadsPerTile))

-- | In place of queueRasterJobs (CallKernels.hs:218-242): BuffersInCommon become one
-- gudni_upload_common call, then every job is rasterized into the host bitmap.
queueRasterJobsCUDA :: MonadIO m => CudaRasterizer -> CInt -> RasterParams token -> [RasterJob] -> m ()
queueRasterJobsCUDA r frameCount params jobs = liftIO $ do
  let target = params ^. rpTarget
      V2 w h = targetArea target
  uploadCommon r params
  case targetBuffer target of
    HostBitmapTarget out ->
      with (params ^. rpSubstanceState . suBackgroundColor) $ \bg ->
        forM_ (zip jobs [0 ..]) $ \(job, jobIndex) ->
          rasterJobCUDA r job (V2 w h) (computeDepthOf params) frameCount jobIndex (castPtr bg) out
    GLTextureTarget _ -> error "GLTextureTarget not implemented"  -- as in the reference

-- | The same frame into a headless target (Graphics.Gudni.CUDA.DrawTarget): a host
-- bitmap through the blocking call, or a device buffer through the stream-ordered
-- one, waited for at the end so that errors are reported here.
queueRasterJobsHeadless :: MonadIO m => CudaRasterizer -> CInt -> RasterParams token -> HeadlessTarget
                        -> [RasterJob] -> m ()
queueRasterJobsHeadless r@(CudaRasterizer ctx) frameCount params target jobs = liftIO $ do
  let area = headlessArea target
      depth = computeDepthOf params
  uploadCommon r params
  with (params ^. rpSubstanceState . suBackgroundColor) $ \bg ->
    case headlessBuffer target of
      HostBitmap out ->
        forM_ (zip jobs [0 ..]) $ \(job, jobIndex) ->
          rasterJobCUDA r job area depth frameCount jobIndex (castPtr bg) out
      DeviceBitmap out stream -> do
        forM_ (zip jobs [0 ..]) $ \(job, jobIndex) ->
          rasterJobDevice r job area depth frameCount jobIndex (castPtr bg) out stream
        check ctx =<< c_syncStatus ctx

-- | Pictures kept on the device across frames: the packed picture pile (makePictData
-- over every usage the application will make) and the random field, uploaded once.
residentPictures :: CudaRasterizer -> Pile Word8 -> VS.Vector CFloat -> IO ()
residentPictures (CudaRasterizer ctx) pictData randoms = do
  check ctx =<< c_uploadPictures ctx (_pileData pictData) (fromIntegral (pictData ^. pileSize))
  VS.unsafeWith randoms $ \p -> check ctx =<< c_uploadRandomField ctx p

-- | Per frame with resident pictures: geometry, substances and the usages (offsets
-- into the resident pile, checked against it by the library).
uploadFrameCUDA :: CudaRasterizer -> RasterParams token
                -> Pile (PictureUsage PictureMemoryReference SubSpace) -> IO ()
uploadFrameCUDA (CudaRasterizer ctx) params pictUsage = do
  let geo  = params ^. rpGeometryState . geoGeometryPile
      subs = params ^. rpSubstanceState . suSubstancePile
  check ctx =<< c_uploadFrame ctx (_pileData geo) (fromIntegral (geo ^. pileSize))
                                  (castPtr (_pileData subs)) (fromIntegral (subs ^. pileSize))
                                  (castPtr (_pileData pictUsage)) (fromIntegral (pictUsage ^. pileSize))
                                  nullPtr 0
