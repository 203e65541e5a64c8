// TrainingLoss (src/trainingLoss.ts:16-130) over the addon: 0.8 L1 + 0.2 (1 -
// SSIM) of a render against an rgba8 photo, and its per-pixel gradient.
// Untested: node is absent here.
import { native, NativeBuffer, NativeDevice } from './native';

export class TrainingLoss {
  readonly pixelGrads: NativeBuffer;
  private readonly handle: unknown;

  constructor(device: NativeDevice, width: number, height: number) {
    this.handle = native.lossCreate(device.handle, width, height);
    this.pixelGrads = new NativeBuffer(native.lossPixelGrads(this.handle));
  }

  encode(_encoder: unknown, rendered: NativeBuffer, target: NativeBuffer): void {
    native.lossEncode(this.handle, rendered.handle, target.handle);
  }

  async read(): Promise<number> {
    return native.lossRead(this.handle);
  }

  destroy(): void {
    native.lossDestroy(this.handle);
  }
}
