/*
 * CudaRendererKernel - the Java side of the JNI binding to the GB300 renderer core (libdfpt.so).
 *
 * Not compiled here: neither image of this project has a JDK. The class is written against
 * Dayflower's own sources (org.dayflower.pathtracer.*) and the Aparapi 1.x Kernel it already
 * builds on (com.amd.aparapi), and its native half, dfpt_jni.c, is compiled and tested in this
 * repository against a stand-in of jni.h and a fake JNIEnv.
 *
 * Drop-in: it extends AbstractRendererKernel and implements every abstract method of that class
 * (AbstractRendererKernel.java:364, 580-726) the way GPURendererKernel does (GPURendererKernel.java:
 * 244-569), but the scene lives in GPU memory owned by the core: the arrays are handed over once in
 * update(), and every put() of the reference becomes one native call. DayflowerApplication changes
 * in one line (DayflowerApplication.java:327):
 *
 *     this.abstractRendererKernel = new CudaRendererKernel(this.sceneLoader);
 *
 * Its render loop (DayflowerApplication.java:853-855) keeps calling execute(range),
 * clearFilmFlags() and get(pixels1); this class overrides Aparapi's execute(Range), get(byte[]),
 * put(...) and dispose() so that none of them reaches Aparapi's OpenCL runtime. If an Aparapi build
 * declares any of them final, the same bodies go into methods of their own (render(),
 * readImage(byte[])) and those three lines call them instead.
 *
 * Build of the native half (a JDK's headers; libdfpt.so from this repository's build):
 *     gcc -O2 -shared -fPIC -I"$JAVA_HOME/include" -I"$JAVA_HOME/include/linux" -I include \
 *         dayflower-path-tracer_gb300/jni/dfpt_jni.c -L dayflower-path-tracer_gb300/dfpt -ldfpt \
 *         -Wl,-rpath,'$ORIGIN' -o libdfpt_jni.so
 * and run the JVM with -Djava.library.path pointing at the folder that holds both libraries.
 */
package org.dayflower.pathtracer.kernel;

import java.util.List;
import java.util.Objects;

import org.dayflower.pathtracer.scene.Camera;
import org.dayflower.pathtracer.scene.Primitive;
import org.dayflower.pathtracer.scene.Scene;
import org.dayflower.pathtracer.scene.Sky;
import org.dayflower.pathtracer.scene.Surface;
import org.dayflower.pathtracer.scene.compiler.CompiledScene;
import org.dayflower.pathtracer.scene.loader.SceneLoader;
import org.dayflower.pathtracer.scene.material.ClearCoatMaterial;
import org.dayflower.pathtracer.scene.material.GlassMaterial;
import org.dayflower.pathtracer.scene.material.LambertianMaterial;
import org.dayflower.pathtracer.scene.material.PhongMaterial;
import org.dayflower.pathtracer.scene.material.ReflectionMaterial;
import org.macroing.math4j.Matrix44F;

import com.amd.aparapi.Kernel;
import com.amd.aparapi.Range;

public final class CudaRendererKernel extends AbstractRendererKernel {
	static {
		System.loadLibrary("dfpt_jni");
	}

	/* Bits of the sky flags argument: dfpt_sky.is_sky_active and is_sun_active. */
	private static final int SKY_FLAG_SKY = 1;
	private static final int SKY_FLAG_SUN = 2;

	/* Material cycle of togglePrimitiveMaterial (GPURendererKernel.java:322-328). */
	private static final int[] MATERIALS = {
		ClearCoatMaterial.TYPE,
		GlassMaterial.TYPE,
		LambertianMaterial.TYPE,
		PhongMaterial.TYPE,
		ReflectionMaterial.TYPE
	};

	private final float[] primitivesObjectToWorld;
	private final float[] primitivesWorldToObject;
	private final float[] surfaces;
	private final int[] primitives;
	private final int[] paramInts = new int[9];
	private final float[] paramFloats = new float[6];
	private int[] primitiveOffsets;
	private int selectedPrimitiveIndex = -1;
	private int selectedPrimitiveOffset = -1;
	private int skyFlags = SKY_FLAG_SKY | SKY_FLAG_SUN;
	private long handle;

	public CudaRendererKernel(final SceneLoader sceneLoader) {
		super(sceneLoader);

		final CompiledScene compiledScene = getCompiledScene();

//		The camera writes its state into the compiled scene's camera array, as GPURendererKernel's constructor sets up (GPURendererKernel.java:166-170).
		getScene().getCamera().setArray(compiledScene.getCamera());

		this.primitives = compiledScene.getPrimitives();
		this.primitivesObjectToWorld = compiledScene.getPrimitivesObjectToWorld();
		this.primitivesWorldToObject = compiledScene.getPrimitivesWorldToObject();
		this.surfaces = compiledScene.getSurfaces();
	}

	////////////////////////////////////////////////////////////////////////////////////////////////////

	/* Aparapi calls run() per work item; this kernel's work runs in libdfpt, so Aparapi never runs it. */
	@Override
	public void run() {

	}

	/* Replaces the Aparapi launch of GPURendererKernel.run() (DayflowerApplication.java:853): one pass
	 * of one sample per pixel, the film accumulated and the BGRA8 image resolved on the GPU. A
	 * clear() since the last frame restarts the film, as FILM_FLAG_CLEAR does
	 * (AbstractImageKernel.java:119-121, 337). */
	@Override
	public synchronized Kernel execute(final Range range) {
		requireHandle();

		if((this.filmFlags & 1) != 0) {
			nativeClear(this.handle);
		}

		pushParams();
		nativeRender(this.handle, 1);

		return this;
	}

	/* Replaces Kernel.get(byte[]) of the image (DayflowerApplication.java:855): the BGRA8 image of the
	 * last pass, written straight into the array. */
	@Override
	public Kernel get(final byte[] array) {
		requireHandle();

		nativeReadBgra8(this.handle, Objects.requireNonNull(array, "array == null"));

		return this;
	}

	/* The arrays live on the GPU from update() on: Aparapi's put() has nothing to copy. */
	@Override
	public Kernel put(final byte[] array) {
		return this;
	}

	@Override
	public Kernel put(final double[] array) {
		return this;
	}

	@Override
	public Kernel put(final float[] array) {
		return this;
	}

	@Override
	public Kernel put(final int[] array) {
		return this;
	}

	/* Replaces Kernel.dispose() (DayflowerApplication.java:502): frees the scene and the film on the GPU. */
	@Override
	public synchronized void dispose() {
		if(this.handle != 0L) {
			nativeDestroy(this.handle);

			this.handle = 0L;
		}
	}

	/* GPURendererKernel.java:244-246. */
	@Override
	public int getSelectedPrimitiveIndex() {
		return this.selectedPrimitiveIndex;
	}

	/* GPURendererKernel.java:314-342: the next material of the cycle for the selected primitive's
	 * surface, then the surfaces array to the GPU. */
	@Override
	public void togglePrimitiveMaterial() {
		final int selectedPrimitiveOffset = this.selectedPrimitiveOffset;

		if(selectedPrimitiveOffset != -1) {
			final int surfacesOffset = this.primitives[selectedPrimitiveOffset + Primitive.RELATIVE_OFFSET_SURFACE_OFFSET];
			final int oldMaterialOrdinal = (int)(this.surfaces[surfacesOffset + Surface.RELATIVE_OFFSET_MATERIAL]) - 1;

			if(oldMaterialOrdinal >= 0 && oldMaterialOrdinal < MATERIALS.length) {
				this.surfaces[surfacesOffset + Surface.RELATIVE_OFFSET_MATERIAL] = MATERIALS[(oldMaterialOrdinal + 1) % MATERIALS.length];

				requireHandle();

				nativeSetSurfaces(this.handle, this.surfaces);

				setChanged(true);
			}
		}
	}

	/* GPURendererKernel.java:351-369: the primitive offset under (x, y) from the last pass's first hits. */
	@Override
	public void togglePrimitiveSelection(final int x, final int y) {
		requireHandle();

		final int index = y * getResolutionX() + x;
		final int[] primitiveOffsets = this.primitiveOffsets;

		nativeReadPrimitiveOffsets(this.handle, primitiveOffsets);

		if(index >= 0 && index < primitiveOffsets.length) {
			final int primitiveOffset = primitiveOffsets[index];

			if(primitiveOffset == this.selectedPrimitiveOffset) {
				this.selectedPrimitiveIndex = -1;
				this.selectedPrimitiveOffset = -1;
			} else {
				this.selectedPrimitiveIndex = primitiveOffset / Primitive.SIZE;
				this.selectedPrimitiveOffset = primitiveOffset;
			}
		}
	}

	/* GPURendererKernel.java:375-383. */
	@Override
	public void toggleSky() {
		this.skyFlags ^= SKY_FLAG_SKY;

		pushSky();
		setChanged(true);
	}

	/* GPURendererKernel.java:389-397. */
	@Override
	public void toggleSun() {
		this.skyFlags ^= SKY_FLAG_SUN;

		pushSky();
		setChanged(true);
	}

	/* GPURendererKernel.java:411-449: the resolution and image array as the reference keeps them, then
	 * the compiled scene, the sky and the film handed to the core once (its 19 put() calls). */
	@Override
	public void update(final int resolutionX, final int resolutionY, final byte[] imageDataByte, final int localSize) {
		update(resolutionX, resolutionY, imageDataByte);

		dispose();

		final CompiledScene c = getCompiledScene();
		final Sky sky = getSky();

		this.primitiveOffsets = new int[resolutionX * resolutionY];
		this.handle = nativeCreate(c.getPoint2Fs(), c.getPoint3Fs(), c.getVector3Fs(), c.getPlanes(), c.getSpheres(), c.getTerrains(), c.getTriangles(), c.getBoundingVolumeHierarchies(), c.getTextures(), c.getSurfaces(), c.getPrimitives(), c.getPrimitivesObjectToWorld(), c.getPrimitivesWorldToObject(), c.getCamera(), skyDoubles(sky), skyFloats(sky), this.skyFlags, resolutionX, resolutionY, System.nanoTime());

		pushParams();

//		The launch structure of execute()'s one-pass renders, picked once for this scene and size; the
//		film and the random streams stay as they were.
		nativeTuneFrame(this.handle, 8);
	}

	/* GPURendererKernel.java:455-461: the camera writes its 19 floats into the compiled scene's array. */
	@Override
	public void updateCamera() {
		final Camera camera = getCamera();

		camera.update();

		requireHandle();

		nativeSetCamera(this.handle, getCompiledScene().getCamera());
	}

	/* GPURendererKernel.java:467-521: both matrices of every primitive, row by row. */
	@Override
	public void updatePrimitives() {
		final Scene scene = getScene();

		if(scene.isPrimitiveUpdateRequired()) {
			final List<Primitive> primitives = scene.getPrimitives();

			for(int i = 0; i < primitives.size(); i++) {
				final Primitive primitive = primitives.get(i);

				primitive.update();

				copyMatrix(primitive.getTransform().getObjectToWorld(), this.primitivesObjectToWorld, i * 16);
				copyMatrix(primitive.getTransform().getWorldToObject(), this.primitivesWorldToObject, i * 16);
			}

			requireHandle();

			nativeSetTransforms(this.handle, this.primitivesObjectToWorld, this.primitivesWorldToObject, primitives.size());

			setChanged(true);
		}
	}

	/* GPURendererKernel.java:527-569. */
	@Override
	public void updateSunAndSky() {
		pushSky();
		setChanged(true);
	}

	////////////////////////////////////////////////////////////////////////////////////////////////////

	private void pushParams() {
		final int[] i = this.paramInts;
		final float[] f = this.paramFloats;

		i[0] = this.rendererType;
		i[1] = this.toneMapperType;
		i[2] = this.shaderType;
		i[3] = this.rendererNormalMapping;
		i[4] = this.rendererWireframes;
		i[5] = this.rendererPTRayDepthMaximum;
		i[6] = this.rendererPTRayDepthRussianRoulette;
		i[7] = getGlobalOctaves();
		i[8] = this.selectedPrimitiveOffset;

		f[0] = this.toneMapperExposure;
		f[1] = this.rendererAOMaximumDistance;
		f[2] = getGlobalAmplitude();
		f[3] = getGlobalFrequency();
		f[4] = getGlobalGain();
		f[5] = getGlobalLacunarity();

//		The native side compares with the values it holds and uploads only a change.
		nativeSetParams(this.handle, i, f);
	}

	private void pushSky() {
		requireHandle();

		final Sky sky = getSky();

		nativeSetSky(this.handle, skyDoubles(sky), skyFloats(sky), this.skyFlags);
	}

	private void requireHandle() {
		if(this.handle == 0L) {
			throw new IllegalStateException("update(resolutionX, resolutionY, imageDataByte, localSize) has not been called");
		}
	}

	/* dfpt_sky's doubles: Perez coefficients (relative luminance, x, y: 5 each), then the zenith's
	 * relative luminance, x and y (Sky.java:142-194). */
	private static double[] skyDoubles(final Sky sky) {
		final double[] d = new double[18];

		System.arraycopy(sky.getPerezRelativeLuminance(), 0, d, 0, 5);
		System.arraycopy(sky.getPerezX(), 0, d, 5, 5);
		System.arraycopy(sky.getPerezY(), 0, d, 10, 5);

		d[15] = sky.getZenithRelativeLuminance();
		d[16] = sky.getZenithX();
		d[17] = sky.getZenithY();

		return d;
	}

	/* dfpt_sky's floats: theta, the basis u, v, w, the sun direction in the sky basis, the sun direction
	 * in world space and the sun origin (Sky.java:106-140, 205-212). */
	private static float[] skyFloats(final Sky sky) {
		return new float[] {
			sky.getTheta(),
			sky.getOrthoNormalBasis().u.x, sky.getOrthoNormalBasis().u.y, sky.getOrthoNormalBasis().u.z,
			sky.getOrthoNormalBasis().v.x, sky.getOrthoNormalBasis().v.y, sky.getOrthoNormalBasis().v.z,
			sky.getOrthoNormalBasis().w.x, sky.getOrthoNormalBasis().w.y, sky.getOrthoNormalBasis().w.z,
			sky.getSunDirection().x, sky.getSunDirection().y, sky.getSunDirection().z,
			sky.getSunDirectionWorld().x, sky.getSunDirectionWorld().y, sky.getSunDirectionWorld().z,
			sky.getSunOrigin().x, sky.getSunOrigin().y, sky.getSunOrigin().z
		};
	}

	private static void copyMatrix(final Matrix44F m, final float[] out, final int offset) {
		out[offset +  0] = m.element11;
		out[offset +  1] = m.element12;
		out[offset +  2] = m.element13;
		out[offset +  3] = m.element14;
		out[offset +  4] = m.element21;
		out[offset +  5] = m.element22;
		out[offset +  6] = m.element23;
		out[offset +  7] = m.element24;
		out[offset +  8] = m.element31;
		out[offset +  9] = m.element32;
		out[offset + 10] = m.element33;
		out[offset + 11] = m.element34;
		out[offset + 12] = m.element41;
		out[offset + 13] = m.element42;
		out[offset + 14] = m.element43;
		out[offset + 15] = m.element44;
	}

	////////////////////////////////////////////////////////////////////////////////////////////////////

//	The native half (dfpt_jni.c). Every failure of the core throws: IllegalArgumentException for
//	invalid arguments or scene arrays, OutOfMemoryError when the GPU is out of memory,
//	IllegalStateException for CUDA errors and timeouts, NullPointerException for a null array.

	private static native long nativeCreate(float[] point2Fs, float[] point3Fs, float[] vector3Fs, int[] planes, float[] spheres, float[] terrains, int[] triangles, int[] boundingVolumeHierarchies, float[] textures, float[] surfaces, int[] primitives, float[] primitivesObjectToWorld, float[] primitivesWorldToObject, float[] camera, double[] skyDoubles, float[] skyFloats, int skyFlags, int resolutionX, int resolutionY, long seed);

	private static native void nativeDestroy(long handle);

	private static native void nativeSetParams(long handle, int[] paramInts, float[] paramFloats);

	private static native void nativeClear(long handle);

	private static native void nativeRender(long handle, int passes);

	private static native void nativeTuneFrame(long handle, int frames);

	private static native void nativeReadBgra8(long handle, byte[] bgra);

	private static native void nativeReadPrimitiveOffsets(long handle, int[] primitiveOffsets);

	private static native void nativeSetCamera(long handle, float[] camera);

	private static native void nativeSetTransforms(long handle, float[] objectToWorld, float[] worldToObject, int primitiveCount);

	private static native void nativeSetSurfaces(long handle, float[] surfaces);

	private static native void nativeSetSky(long handle, double[] skyDoubles, float[] skyFloats, int skyFlags);
}
