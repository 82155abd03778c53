// pbf.ts - the reference's simulator and renderer classes over the
// pbf_gb300 Node-API addon (pbf_addon.cc), for a Node host that keeps the
// reference's controller code: the method names, arguments and thrown
// errors of src/simulator/SPH.ts, src/simulator/PBF/PBFConfig.ts,
// src/simulator/PBF/PBF.ts and src/renderer/filteredParticleFluid/fluid.ts.
// WebGPU objects do not cross this boundary: `run()` needs no command
// encoder, and the `position` buffer is read into a Float32Array
// (`readPositions`) or consumed on the device by the CUDA renderer.

// eslint-disable-next-line @typescript-eslint/no-var-requires
const addon = require('./build/Release/pbf_gb300.node');

export interface Vec3Like { x: number; y: number; z: number; }

// The parts of a three.js Mesh that SPH.voxelizeMesh reads.
export interface MeshLike {
  geometry: {
    getAttribute(name: 'position'): { array: ArrayLike<number> };
    index: { array: ArrayLike<number> } | null;
  };
  matrixWorld: { elements: ArrayLike<number> };
  updateMatrixWorld(force?: boolean): void;
}

// The parts of a three.js PerspectiveCamera that the camera uniform reads
// (src/common/globalResource.ts:94-109, 165-181).
export interface CameraLike {
  position: Vec3Like;
  matrixWorld: { elements: ArrayLike<number> };
  matrixWorldInverse: { elements: ArrayLike<number> };
  projectionMatrix: { elements: ArrayLike<number> };
  fov: number;
  aspect: number;
  near: number;
  far: number;
}

export interface PBFOptions {
  iteration: number;
  XSPH: number;
  vorticity: number;
  surfaceTension: number;
  gravity: number;
}

export interface SimulatorConfig {
  particleRadius?: number;  // r (0.006)
  kernelRadius?: number;    // h (0.025)
  restDensity?: number;     // rho0 (1000)
  timeStep?: number;        // dt of one substep (1/300)
  stepCount?: number;       // substeps per frame (1)
  maxParticles?: number;    // capacity (SPH.MAX_PARTICLE_NUM)
  maxNeighbors?: number;
  domainMin?: [number, number, number];
  domainMax?: [number, number, number];
  fastMath?: boolean;       // FMA contraction (default); false = bit-exact with the CPU restatement
}

const v3 = (v: Vec3Like): number[] => [v.x, v.y, v.z];

// SPH + PBFConfig + PBF (constructor and initResource in one step).
export class PBF {
  public readonly handle: unknown;
  public readonly stepCount: number;

  constructor(config: SimulatorConfig = {}) {
    this.handle = addon.create(config);
    this.stepCount = config.stepCount ?? 1;
    addon.setPaused(this.handle, true);  // SPH.ts:45: a new simulator is paused
  }

  public get particleCount(): number { return addon.particleCount(this.handle); }

  public get pause(): boolean { return addon.isPaused(this.handle); }
  public set pause(p: boolean) { addon.setPaused(this.handle, p); }

  // SPH.ts:82-84
  public switch() { this.pause = !this.pause || this.particleCount === 0; }
  public stop() { this.pause = true; }
  public start() { this.pause = this.particleCount === 0; }

  // SPH.ts:99-187: append lattice points; setParticlePosition uploads them.
  public voxelizeCube(min: Vec3Like, max: Vec3Like): number {
    return addon.voxelizeCube(this.handle, v3(min), v3(max));
  }
  public voxelizeSphere(center: Vec3Like, radius: number): number {
    return addon.voxelizeSphere(this.handle, v3(center), radius);
  }
  public voxelizeMesh(mesh: MeshLike): number {
    mesh.updateMatrixWorld();
    const pos = Float32Array.from(mesh.geometry.getAttribute('position').array);
    const index = mesh.geometry.index ? Uint32Array.from(mesh.geometry.index.array) : null;
    return addon.voxelizeMesh(this.handle, pos, index, Float64Array.from(mesh.matrixWorld.elements));
  }
  public setParticlePosition() { addon.setParticlePosition(this.handle); }

  // PBFConfig.ts:31-46, 64-66
  public setConfig(conf: PBFOptions) { addon.setConfig(this.handle, conf); }
  public optionsChange(e: { object: PBFOptions }) { this.setConfig(e.object); }

  // PBF.ts:71-94
  public reset() { addon.reset(this.handle); }
  public setBoundaryData(data: string) { addon.setBoundaryData(this.handle, data); }

  // PBF.run (one substep) and the controller's frame of stepCount substeps
  // (src/controller.ts:375-376); both do nothing while paused.
  public run() { addon.run(this.handle); }
  public frame(frames = 1) { addon.step(this.handle, frames); }
  // PBF.runTimestamp: [integrate, neighbour search, constraints, non-pressure] ms
  public runTimestamp(): number[] { return addon.runTimestamp(this.handle); }

  // The `position` buffer (x, y, z, density per particle).
  public readPositions(out?: Float32Array): Float32Array {
    const dst = out ?? new Float32Array(4 * this.particleCount);
    addon.copyPositions(this.handle, dst);
    return dst;
  }
  // The same, written while the next frames run; complete after synchronize().
  public readPositionsAsync(out: Float32Array) { addon.copyPositionsAsync(this.handle, out); }
  public synchronize() { addon.synchronize(this.handle); }
  public metrics() { return addon.metrics(this.handle); }

  public update() { }
  public destroy() { addon.destroy(this.handle); }
}

export interface RenderingOptions {
  mode?: number;
  filterSize?: number;
  particleRadius?: number;
  opacity?: number;
  tintColor?: [number, number, number];  // 0..255
}

// FilteredParticleFluid's depth and volume maps (fluid.ts:77-160), computed
// on the GPU from the simulator's positions.
export class FilteredParticleFluid {
  public readonly handle: unknown;

  constructor(private simulator: PBF, public readonly width: number, public readonly height: number) {
    this.handle = addon.rendererCreate(width, height);
  }

  public setConfig(options: RenderingOptions) { addon.rendererSetConfig(this.handle, options); }

  public setCamera(camera: CameraLike) {
    const h = 2.0 * camera.near * Math.tan((Math.PI / 180.0) * 0.5 * camera.fov);
    addon.rendererSetCamera(this.handle, {
      position: v3(camera.position),
      view: Array.from(camera.matrixWorldInverse.elements),
      viewInverse: Array.from(camera.matrixWorld.elements),
      projection: Array.from(camera.projectionMatrix.elements),
      params: [camera.aspect * h / camera.near, -h / camera.near,
        (camera.far - camera.near) / (camera.near * camera.far), 1.0 / camera.far],
    });
  }

  // ParicleRasterizer.execute + TextureFilter.execute (fluid.ts:150-160)
  public render() { addon.renderSimulation(this.handle, this.simulator.handle); }

  public depthMap(out?: Float32Array): Float32Array {
    const dst = out ?? new Float32Array(this.width * this.height);
    addon.copyMap(this.handle, 0, dst);
    return dst;
  }
  public volumeMap(out?: Float32Array): Float32Array {
    const [w, h] = addon.mapSize(this.handle, 1);
    const dst = out ?? new Float32Array(w * h);
    addon.copyMap(this.handle, 1, dst);
    return dst;
  }

  public destroy() { addon.rendererDestroy(this.handle); }
}
