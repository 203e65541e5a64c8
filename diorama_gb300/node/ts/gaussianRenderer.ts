// GaussianRenderer (src/gaussianRenderer.ts:55-311) over the addon. The encoder
// arguments of the WebGPU version are accepted and ignored: work is enqueued on
// the device's in-order stream when encode is called, and runs in call order as
// WebGPU submissions do. Untested: node is absent here.
import { native, NativeBuffer, NativeDevice } from './native';

export interface CameraData {
  view: Float32Array;
  proj: Float32Array;
  viewport: [number, number];
}

export type RGB = [number, number, number];

export class GaussianRenderer {
  readonly handle: unknown;

  constructor(device: NativeDevice, options: { initialPairCapacity?: number } = {}, handle?: unknown) {
    this.handle = handle ?? native.rendererCreate(device.handle, options.initialPairCapacity ?? 0);
  }

  setGaussians(data: Float32Array, sh?: { rest: Float32Array; degree: number }): void {
    native.rendererSetGaussians(this.handle, data, sh);
  }

  setShDegree(degree: number): void {
    native.rendererSetShDegree(this.handle, degree);
  }

  encode(_encoder: unknown, target: NativeBuffer | undefined, camera: CameraData, background: RGB): void {
    native.rendererEncode(this.handle, target?.handle, camera, background);
  }

  encodeBackward(_encoder: unknown, pixelGrads: NativeBuffer): void {
    native.rendererEncodeBackward(this.handle, pixelGrads.handle);
  }

  // Reads back the frame's pair count and grows the pair buffers if it did not fit.
  async afterSubmit(): Promise<void> {
    native.rendererAfterSubmit(this.handle);
  }

  private buffer(name: string): NativeBuffer | undefined {
    const h = native.rendererBuffer(this.handle, name);
    return h === undefined ? undefined : new NativeBuffer(h);
  }
  get splatBuffer() {
    return this.buffer('splat');
  }
  get gaussianBuffer() {
    return this.buffer('gaussian');
  }
  get shBuffer() {
    return this.buffer('sh');
  }
  get pixelBuffer() {
    return this.buffer('pixel');
  }
  get pixelLastBuffer() {
    return this.buffer('pixelLast');
  }
  get gradients() {
    return { gaussians: this.buffer('gradGaussians'), sh: this.buffer('gradSh'), splats: this.buffer('gradSplats') };
  }

  destroy(): void {
    native.rendererDestroy(this.handle);
  }
}
