{-# LANGUAGE BangPatterns        #-}
{-# LANGUAGE MagicHash           #-}
{-# LANGUAGE RecordWildCards     #-}
{-# LANGUAGE ScopedTypeVariables #-}

{- |
Drop-in replacement for shapes' @Physics.Engine.Main@
(shapes/src/Physics/Engine/Main.hs) that steps the world on a GB300 through
libshapes_gpu.so (include/shapes_gpu.h).  The exported names and the types of
the stepping API are the reference's: 'EngineConfig', 'EngineST', 'initEngine',
'changeScene', 'updateWorld', 'stepWorld', 'runEngine', 'runWorld'.  The
second component of 'EngineState' holds the GPU handle instead of the
contact cache (the cache lives on the device, carried between steps exactly
as the reference's 'EngineCache' is; 'engineCache' reads it back).

What stays on the host: the 'World' (labels, materials, shapes, body state),
kept in step with the device after every 'updateWorld' / 'stepWorld' so that
callers reading it (the demo's drawing and queries) see the stepped state.
What crosses the FFI: body state as ten SoA double arrays, hull vertices in
local coordinates ('_hullLocalVertices'), a circle as one point (radius, 0).
'External' is a closure and cannot cross; 'initEngine' probes it and accepts
'constantAccel' (World/External.hs:23-28) and @const id@, else it fails.

Requirements: the scene's world has no empty slots (as 'makeWorld' /
'fromList' builds it); slot i is body i of the device world, so contact keys
('ObjectFeatureKey') are the reference's.  The solver sweep count is the
reference's 2 (Engine/Main.hs:81-82) with warm starting on.

Not compiled in this repository (no GHC here).  Build with the reference's
stack project plus Physics/Engine/GPU/FFI.hs, linking -lshapes_gpu.
-}
module Physics.Engine.Main ( module Physics.Engine.Main
                           , module Physics.Engine
                           ) where

import           Control.Monad                (forM, forM_, when)
import           Control.Monad.Reader
import           Control.Monad.ST
import           Control.Monad.ST.Unsafe      (unsafeIOToST)
import           Control.Monad.State.Strict
import           Data.Array                   (elems)
import           Data.Int                     (Int32, Int64)
import           Data.IORef
import           Foreign
import           Foreign.C.String             (peekCString)
import           Foreign.C.Types
import           GHC.Exts                     (Double (D#), Double#)

import           Physics.Constraint           (InvMass2 (..), PhysicalObj (..))
import           Physics.Constraints.Contact  (ObjectFeatureKey (..))
import           Physics.Contact              (Shape (..))
import           Physics.Contact.Circle       (Circle (..))
import           Physics.Contact.ConvexHull   (ConvexHull (..))
import           Physics.Contact.Types        (ContactBehavior (..))
import           Physics.Engine
import           Physics.Engine.GPU.FFI
import           Physics.Linear               (P2 (..), V2 (..))
import           Physics.Scenes.Scene
import           Physics.World
import qualified Utils.EmptiesVector          as E

-- | The device world and the External as data.
data GpuEngine = GpuEngine
  { geBatch  :: !(ForeignPtr ShapesBatch)
  , geExt    :: !(Int32, Double, Double) -- ^ SHAPES_EXTERNAL_*, acceleration x, y
  , geBodies :: !Int
  }

type EngineState label s = (World s label, GpuEngine, External)
data EngineConfig = EngineConfig
  { _engineTimestep :: Double
  , _engineContactBeh :: ContactBehavior
  } deriving (Show)
type EngineST label s = ReaderT EngineConfig (StateT (EngineState label s) (ST s))

-- | Reference: initEngine (Engine/Main.hs:43-46).  Uploads the scene's world
-- (shapes_batch_create); the contact cache starts empty, as MV.new 0 does.
initEngine :: Scene s label -> ST s (EngineState label s)
initEngine Scene{..} = do
  slots <- E.foldM (\acc i -> return (i : acc)) [] (_wEmpties _scWorld)
  let n = length slots
  when (reverse slots /= [0 .. n - 1]) $
    error "Physics.Engine.Main (GPU): the world must have no empty slots (build it with makeWorld)"
  objs <- mapM (readPhysObj _scWorld) [0 .. n - 1]
  mats <- mapM (readMaterial _scWorld) [0 .. n - 1]
  shapes <- mapM (readShape _scWorld) [0 .. n - 1]
  ext <- either error return (probeExternal _scExts)
  batch <- unsafeIOToST (createBatch objs mats shapes)
  return (_scWorld, GpuEngine batch ext n, _scExts)

-- | Reference: changeScene (Engine/Main.hs:48-51).  The previous handle is
-- freed by its finalizer.
changeScene :: Scene s label -> EngineST label s ()
changeScene scene = do
  eState <- lift . lift $ initEngine scene
  put eState

-- | Reference: updateWorld (Engine/Main.hs:71-84), one step on the device:
-- broadphase, gravity, contacts, warm start from the device cache, 2 sweeps,
-- integration and re-posing.
updateWorld :: EngineST label s ()
updateWorld = stepWorld 1

-- | Reference: stepWorld (Engine/Main.hs:88-89) = replicateM_ steps
-- updateWorld; here one FFI call steps the device world `steps` times (the
-- same results: nothing on the host changes between the steps).
stepWorld :: Int -> EngineST label s ()
stepWorld steps = do
  EngineConfig{..} <- ask
  (world, eng, _) <- get
  let ContactBehavior beta slop = _engineContactBeh
      (ext, ax, ay) = geExt eng
      cfg = Config (realToFrac _engineTimestep) (realToFrac beta) (realToFrac slop) (realToFrac ax)
                   (realToFrac ay) 2 1 ext 0
  lift . lift $ do
    objs <- mapM (readPhysObj world) [0 .. geBodies eng - 1]
    mats <- mapM (readMaterial world) [0 .. geBodies eng - 1]
    objs' <- unsafeIOToST $ withForeignPtr (geBatch eng) $ \b -> do
      withBodies objs mats $ \bp -> c_batch_set_bodies b bp >>= check "shapes_batch_set_bodies"
      with cfg $ \cp -> c_batch_step b cp (fromIntegral steps) >>= check "shapes_batch_step"
      downloadBodies b (geBodies eng)
    forM_ (zip [0 ..] objs') $ uncurry (updatePhysObj world)
    moveShapes world

-- | Reference: runEngine (Engine/Main.hs:91-95).
runEngine :: Double -> Scene s label -> EngineST label s b -> ST s b
runEngine dt scene@Scene{..} action = do
  state' <- initEngine scene
  evalStateT (runReaderT action engineConfig) state'
  where engineConfig = EngineConfig dt _scContactBeh

-- | Reference: runWorld (Engine/Main.hs:97-98).
runWorld :: Double -> Scene s label -> Int -> ST s ()
runWorld dt scene steps = runEngine dt scene $ stepWorld steps

-- | The device's contact cache (the reference's EngineCache contents), in
-- the reference's order: ((i, j), (feature i, feature j)) and the normal and
-- friction Lagrangians.
engineCache :: EngineST label s [(ObjectFeatureKey Int, (Double, Double))]
engineCache = do
  (_, eng, _) <- get
  lift . lift . unsafeIOToST . withForeignPtr (geBatch eng) $ \b -> do
    n <- alloca $ \np -> c_batch_num_cache b np >>= check "shapes_batch_num_cache" >> peek np
    let m = fromIntegral (n :: Int64)
    allocaArray (4 * max m 1) $ \kp -> allocaArray (2 * max m 1) $ \lp -> alloca $ \wc -> do
      c_batch_get_cache b kp lp n wc >>= check "shapes_batch_get_cache"
      ks <- peekArray (4 * m) kp
      ls <- peekArray (2 * m) lp
      return [ (ObjectFeatureKey (fi i, fi j) (fi fa, fi fb), (realToFrac ln, realToFrac lf))
             | ((i, j, fa, fb), (ln, lf)) <- zip (quads ks) (pairs ls) ]
  where
    fi :: Int32 -> Int
    fi = fromIntegral
    quads (a : b : c : d : r) = (a, b, c, d) : quads r
    quads _ = []
    pairs (a : b : r) = (a, b) : pairs r
    pairs _ = []

-- ---- marshalling -------------------------------------------------------------

check :: String -> CInt -> IO ()
check what rc = when (rc /= statusOk) $ do
  msg <- c_strerror rc >>= peekCString
  ioError (userError (what ++ ": " ++ msg))

fromV2 :: V2 -> (Double, Double)
fromV2 (V2 x y) = (D# x, D# y)

unD :: Double -> Double#
unD (D# d) = d

-- | The External as data: 'constantAccel' a gives v + a*dt to every body with
-- a finite inverse mass; @const id@ changes nothing.  A probe body with
-- velocity (-0, -0) tells them apart (-0 + 0 = +0), a second one checks the
-- dt scaling.
probeExternal :: External -> Either String (Int32, Double, Double)
probeExternal f
  | isNegativeZero ax0 && isNegativeZero ay0 && (bx, by) == (1, -1) = Right (externalNone, 0, 0)
  | bx == 1 + 2 * ax0 && by == -1 + 2 * ay0 = Right (externalConstantAccel, ax0, ay0)
  | otherwise = Left "Physics.Engine.Main (GPU): External must be constantAccel or const id"
  where
    probe v = makePhysicalObj v 0 (0, 0) 0 (1, 1)
    (ax0, ay0) = fromV2 (_physObjVel (f 1 (probe (-0.0, -0.0))))
    (bx, by) = fromV2 (_physObjVel (f 2 (probe (1, -1))))

-- | Ten SoA arrays of the bodies, valid inside the callback.
withBodies :: [PhysicalObj] -> [Material] -> (Ptr Bodies -> IO a) -> IO a
withBodies objs mats k = do
  let col f = map (CDouble . f) objs
      vx o = fst (fromV2 (_physObjVel o))
      vy o = snd (fromV2 (_physObjVel o))
      px o = fst (fromV2 (_physObjPos o))
      py o = snd (fromV2 (_physObjPos o))
      iml o = case _physObjInvMass o of InvMass2 l _ -> D# l
      imr o = case _physObjInvMass o of InvMass2 _ r -> D# r
      mcol f = map (CDouble . f) mats
  withArray (col vx) $ \a -> withArray (col vy) $ \b -> withArray (col _physObjRotVel) $ \c ->
    withArray (col px) $ \d -> withArray (col py) $ \e -> withArray (col _physObjRotPos) $ \f ->
    withArray (col iml) $ \g -> withArray (col imr) $ \h -> withArray (mcol _mMu) $ \i ->
    withArray (mcol _mBounce) $ \j -> with (Bodies a b c d e f g h i j) k

downloadBodies :: Ptr ShapesBatch -> Int -> IO [PhysicalObj]
downloadBodies b n =
  allocaArray n $ \a -> allocaArray n $ \b' -> allocaArray n $ \c -> allocaArray n $ \d ->
  allocaArray n $ \e -> allocaArray n $ \f -> allocaArray n $ \g -> allocaArray n $ \h ->
  allocaArray n $ \i -> allocaArray n $ \j -> do
    with (Bodies a b' c d e f g h i j) $ \bp -> c_batch_get_bodies b bp >>= check "shapes_batch_get_bodies"
    [vx, vy, w, px, py, th, iml, imr] <- mapM (fmap (map realToFrac) . peekArray n) [a, b', c, d, e, f, g, h]
    return [ PhysicalObj (pairToV2 (vx_, vy_)) w_ (pairToV2 (px_, py_)) th_ (InvMass2 (unD l) (unD r))
           | (vx_, vy_, w_, px_, py_, th_, l, r) <- zip8 vx vy w px py th iml imr ]
  where
    zip8 (a : as) (b : bs) (c : cs) (d : ds) (e : es) (f : fs) (g : gs) (h : hs) =
      (a, b, c, d, e, f, g, h) : zip8 as bs cs ds es fs gs hs
    zip8 _ _ _ _ _ _ _ _ = []

-- | shapes_batch_create for one world: SoA bodies, hull vertices in local
-- coordinates (listToHull's order), circles as one point (radius, 0).
createBatch :: [PhysicalObj] -> [Material] -> [Shape] -> IO (ForeignPtr ShapesBatch)
createBatch objs mats shapes = do
  let local (HullShape h) = [ fromV2 v | P2 v <- elems (_hullLocalVertices h) ]
      local (CircleShape c) = [(_circleRadius c, 0)]
      kind (HullShape _) = shapeHull
      kind (CircleShape _) = shapeCircle
      pts = map local shapes
      offs = scanl (+) 0 (map length pts) :: [Int]
      xy = concat [ [CDouble x, CDouble y] | ps <- pts, (x, y) <- ps ]
      n = length objs
  withArray [0, fromIntegral n :: Int32] $ \wo ->
    withArray (map fromIntegral offs :: [Int32]) $ \vo ->
    withArray xy $ \xyp -> withArray (map kind shapes) $ \kp ->
    withBodies objs mats $ \bp -> alloca $ \out -> do
      c_batch_create 1 wo bp vo xyp kp out >>= check "shapes_batch_create"
      peek out >>= newForeignPtr p_batch_destroy
