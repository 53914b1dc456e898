{-# LANGUAGE ForeignFunctionInterface #-}
{- |
Foreign imports of libshapes_gpu.so (include/shapes_gpu.h) for the Haskell
engine shim in Physics/Engine/Main.hs.  Long calls are imported @safe@ so the
RTS keeps running other Haskell threads while the GPU works.

Not compiled in this repository (no GHC here); written against GHC's FFI and
base only.  Link: ghc ... -L<repo>/shapes_gb300/_build -lshapes_gpu
-optl-Wl,-rpath,<repo>/shapes_gb300/_build
-}
module Physics.Engine.GPU.FFI
  ( ShapesBatch
  , Bodies (..)
  , Config (..)
  , statusOk
  , c_batch_create
  , c_batch_step
  , c_batch_get_bodies
  , c_batch_set_bodies
  , c_batch_num_bodies
  , c_batch_num_cache
  , c_batch_get_cache
  , c_batch_set_cache
  , c_strerror
  , p_batch_destroy
  , externalConstantAccel
  , externalNone
  , shapeHull
  , shapeCircle
  ) where

import           Data.Int         (Int32, Int64)
import           Data.Word        (Word8)
import           Foreign
import           Foreign.C.String (CString)
import           Foreign.C.Types

-- | Opaque @shapes_batch@ (one or many independent worlds on the GPU).
data ShapesBatch

-- | @shapes_bodies@: ten pointers to SoA arrays of doubles, in this order.
data Bodies = Bodies
  { bVelX, bVelY, bRotVel, bPosX, bPosY, bRot, bImLin, bImRot, bMu, bBounce :: !(Ptr CDouble) }

instance Storable Bodies where
  sizeOf _ = 10 * sizeOf (undefined :: Ptr CDouble)
  alignment _ = alignment (undefined :: Ptr CDouble)
  peek p = Bodies <$> f 0 <*> f 1 <*> f 2 <*> f 3 <*> f 4 <*> f 5 <*> f 6 <*> f 7 <*> f 8 <*> f 9
    where f = peekElemOff (castPtr p)
  poke p (Bodies a b c d e f g h i j) =
    mapM_ (uncurry (pokeElemOff (castPtr p))) (zip [0 ..] [a, b, c, d, e, f, g, h, i, j])

-- | @shapes_config@: dt, Baumgarte factor, penetration slop, acceleration x/y
-- (five doubles), then sweep count, warm start, external and flags (int32).
data Config = Config
  { cDt, cBaumgarte, cSlop, cAccelX, cAccelY :: !CDouble
  , cIterations, cWarmStart, cExternal, cFlags :: !Int32
  }

instance Storable Config where
  sizeOf _ = 5 * 8 + 4 * 4
  alignment _ = 8
  peek p = Config <$> d 0 <*> d 1 <*> d 2 <*> d 3 <*> d 4 <*> i 0 <*> i 1 <*> i 2 <*> i 3
    where d k = peekByteOff p (8 * k)
          i k = peekByteOff p (40 + 4 * k)
  poke p (Config dt b s ax ay it ws ex fl) = do
    mapM_ (\(k, v) -> pokeByteOff p (8 * k) v) (zip [0 ..] [dt, b, s, ax, ay])
    mapM_ (\(k, v) -> pokeByteOff p (40 + 4 * k) v) (zip [0 ..] [it, ws, ex, fl])

statusOk :: CInt
statusOk = 0

-- | SHAPES_EXTERNAL_CONSTANT_ACCEL / SHAPES_EXTERNAL_NONE
externalConstantAccel, externalNone :: Int32
externalConstantAccel = 1
externalNone = 0

-- | SHAPES_SHAPE_HULL / SHAPES_SHAPE_CIRCLE
shapeHull, shapeCircle :: Word8
shapeHull = 0
shapeCircle = 1

foreign import ccall safe "shapes_batch_create"
  c_batch_create :: Int32 -> Ptr Int32 -> Ptr Bodies -> Ptr Int32 -> Ptr CDouble -> Ptr Word8
                 -> Ptr (Ptr ShapesBatch) -> IO CInt
foreign import ccall safe "shapes_batch_step"
  c_batch_step :: Ptr ShapesBatch -> Ptr Config -> Int32 -> IO CInt
foreign import ccall safe "shapes_batch_get_bodies"
  c_batch_get_bodies :: Ptr ShapesBatch -> Ptr Bodies -> IO CInt
foreign import ccall safe "shapes_batch_set_bodies"
  c_batch_set_bodies :: Ptr ShapesBatch -> Ptr Bodies -> IO CInt
foreign import ccall unsafe "shapes_batch_num_bodies"
  c_batch_num_bodies :: Ptr ShapesBatch -> Ptr Int64 -> IO CInt
foreign import ccall unsafe "shapes_batch_num_cache"
  c_batch_num_cache :: Ptr ShapesBatch -> Ptr Int64 -> IO CInt
foreign import ccall safe "shapes_batch_get_cache"
  c_batch_get_cache :: Ptr ShapesBatch -> Ptr Int32 -> Ptr CDouble -> Int64 -> Ptr Int32 -> IO CInt
foreign import ccall safe "shapes_batch_set_cache"
  c_batch_set_cache :: Ptr ShapesBatch -> Ptr Int32 -> Ptr Int32 -> Ptr CDouble -> IO CInt
foreign import ccall unsafe "shapes_strerror"
  c_strerror :: CInt -> IO CString
foreign import ccall "&shapes_batch_destroy"
  p_batch_destroy :: FunPtr (Ptr ShapesBatch -> IO ())
