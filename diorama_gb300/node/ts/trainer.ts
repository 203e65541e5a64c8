// Trainer (src/trainer.ts:103-446) over the addon, with the reference's
// TrainingSettings and DEFAULT_SETTINGS. step() resolves when the step's work,
// including a densification's readback of the new count, is done on the thread
// pool. Untested: node is absent here.
import { GaussianRenderer, type CameraData, type RGB } from './gaussianRenderer';
import { native, NativeBuffer, NativeDevice } from './native';

export interface TrainingView {
  name: string;
  camera: CameraData;
  image: NativeBuffer; // rgba8 bytes of the viewport's size
}

export interface RawGaussians {
  params: Float32Array;
  sh: Float32Array;
}

export interface TrainingSettings {
  extent: number;
  positionLrSteps: number;
  positionLr: [number, number];
  opacityLr: number;
  scaleLr: number;
  rotationLr: number;
  colorLr: number;
  shLr: number;
  shDegreeInterval: number;
  densifyFrom: number;
  densifyUntil: number;
  densifyInterval: number;
  densifyGradThreshold: number;
  percentDense: number;
  minOpacity: number;
  opacityResetInterval: number;
  background: RGB;
}

export const DEFAULT_SETTINGS: Omit<TrainingSettings, 'extent'> = {
  positionLrSteps: 30_000,
  positionLr: [0.00016, 0.0000016],
  opacityLr: 0.025,
  scaleLr: 0.005,
  rotationLr: 0.001,
  colorLr: 0.0025,
  shLr: 0.0025 / 20,
  shDegreeInterval: 1000,
  densifyFrom: 500,
  densifyUntil: 15_000,
  densifyInterval: 100,
  densifyGradThreshold: 0.0002,
  percentDense: 0.01,
  minOpacity: 0.005,
  opacityResetInterval: 3000,
  background: [0, 0, 0],
};

export class Trainer {
  readonly renderer: GaussianRenderer;
  private readonly handle: unknown;

  constructor(
    device: NativeDevice,
    raw: RawGaussians,
    views: TrainingView[],
    readonly settings: TrainingSettings,
  ) {
    const plain = views.map((v) => ({ camera: v.camera, image: v.image.handle }));
    this.handle = native.trainerCreate(device.handle, raw, plain, settings);
    this.renderer = new GaussianRenderer(device, {}, native.trainerRenderer(this.handle));
  }

  get iteration(): number {
    return native.trainerIteration(this.handle);
  }

  get count(): number {
    return native.trainerCount(this.handle);
  }

  step(): Promise<void> {
    return native.trainerStep(this.handle);
  }

  async lastLoss(): Promise<number> {
    return native.trainerLastLoss(this.handle);
  }

  async exportRaw(): Promise<RawGaussians> {
    return native.trainerExportRaw(this.handle);
  }

  async evaluate(views: TrainingView[], withSsim = true): Promise<{ psnr: number; ssim: number }> {
    const plain = views.map((v) => ({ camera: v.camera, image: v.image.handle }));
    return native.trainerEvaluate(this.handle, plain, withSsim);
  }

  destroy(): void {
    native.trainerDestroy(this.handle);
  }
}
